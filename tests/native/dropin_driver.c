/*
 * dropin_driver.c -- a C caller of the drop-in entry points, linked against
 * libzccl_gpu.so through include/zccl_gpu.h the way a reference caller is
 * (no Python in between).  It follows the reference's codec driver
 * (examples/testfloat_homocompress_fastmode1_arg.c:204-268): compress two
 * arrays, decompress one, add them homomorphically in place, and also runs
 * the allocating and the _record variants.  Outputs go to files in `dir`
 * for the test to compare with the oracle; counts go to stdout as
 * "name value" lines.
 *
 * usage: dropin_driver dir n L eb T     (reads dir/x.f32 and dir/y.f32)
 */
#include <omp.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "zccl_gpu.h"

static void *read_file(const char *dir, const char *name, size_t bytes)
{
    char path[4096];
    snprintf(path, sizeof path, "%s/%s", dir, name);
    FILE *f = fopen(path, "rb");
    if (!f) return NULL;
    void *p = malloc(bytes);
    if (p && fread(p, 1, bytes, f) != bytes) {
        free(p);
        p = NULL;
    }
    fclose(f);
    return p;
}

static int write_file(const char *dir, const char *name, const void *p, size_t bytes)
{
    char path[4096];
    snprintf(path, sizeof path, "%s/%s", dir, name);
    FILE *f = fopen(path, "wb");
    if (!f) return -1;
    const size_t w = fwrite(p, 1, bytes, f);
    fclose(f);
    return w == bytes ? 0 : -1;
}

#define CHECK(what)                                                                      \
    do {                                                                                 \
        int st_ = zccl_gpu_last_status();                                                \
        if (st_ != ZCCL_GPU_OK) {                                                        \
            fprintf(stderr, "%s failed: %s\n", what, zccl_gpu_strerror(st_));            \
            return 1;                                                                    \
        }                                                                                \
    } while (0)

int main(int argc, char **argv)
{
    if (argc != 6) {
        fprintf(stderr, "usage: %s dir n L eb T\n", argv[0]);
        return 2;
    }
    const char *dir = argv[1];
    const size_t n = strtoull(argv[2], NULL, 10);
    const int L = atoi(argv[3]);
    const float eb = strtof(argv[4], NULL);
    const int T = atoi(argv[5]);
    omp_set_num_threads(T);

    float *x = read_file(dir, "x.f32", 4 * n), *y = read_file(dir, "y.f32", 4 * n);
    if (!x || !y) return 2;
    const size_t cap = zccl_gpu_max_stream_bytes(n, L, T) + zccl_gpu_max_stream_bytes(n, L, 1) + 64;
    unsigned char *a = calloc(cap, 1), *b = calloc(cap, 1), *a1 = calloc(cap, 1), *frame = calloc(cap + 16, 1);
    float *dec = calloc(n, sizeof(float)), *dec1 = calloc(n, sizeof(float));
    if (!a || !b || !a1 || !frame || !dec || !dec1) return 2;

    /* the _arg variants, as the reference driver calls them */
    size_t sa = 0, sb = 0, sh = 0;
    ZCCL_float_openmp_threadblock_arg(a, x, &sa, eb, n, L);
    CHECK("compress");
    ZCCL_float_openmp_threadblock_arg(b, y, &sb, eb, n, L);
    CHECK("compress");
    ZCCL_float_decompress_openmp_threadblock_arg(dec, n, eb, L, a);
    CHECK("decompress");
    if (write_file(dir, "a.zc", a, sa) || write_file(dir, "a.dec", dec, 4 * n)) return 3;

    /* the allocating variants give the same bytes and floats */
    size_t sm = 0;
    unsigned char *am = ZCCL_float_openmp_threadblock(x, &sm, eb, n, L);
    CHECK("compress (malloc)");
    float *decm = NULL;
    ZCCL_float_decompress_openmp_threadblock(&decm, n, eb, L, am);
    CHECK("decompress (malloc)");
    printf("malloc_stream_equal %d\n", sm == sa && memcmp(am, a, sa) == 0);
    printf("malloc_floats_equal %d\n", memcmp(decm, dec, 4 * n) == 0);
    free(am);
    free(decm);

    /* the add, in place over its second input (ZCCL_ring_ho.c:281-287), with
     * the branch counters of the _record variant starting from 100 */
    int c1 = 100, c2 = 100, c3 = 100, c4 = 100;
    ZCCL_float_homomophic_add_openmp_threadblock_record(b, &sh, n, eb, L, a, b, &c1, &c2, &c3, &c4);
    CHECK("homomorphic add (record)");
    if (write_file(dir, "h.zc", b, sh)) return 3;
    printf("cases %d %d %d %d\n", c1 - 100, c2 - 100, c3 - 100, c4 - 100);

    /* T = 1: the _record variants' counts and the split variant's frame */
    size_t s1 = 0;
    const size_t cc = ZCCL_float_single_thread_arg_record(a1, x, &s1, eb, n, L);
    CHECK("compress (record)");
    const size_t dc = ZCCL_float_decompress_single_thread_arg_record(dec1, n, eb, L, a1);
    CHECK("decompress (record)");
    if (write_file(dir, "a1.zc", a1, s1) || write_file(dir, "a1.dec", dec1, 4 * n)) return 3;
    printf("compress_count %zu\n", cc);
    printf("decompress_count %zu\n", dc);
    size_t sp = 0;
    ZCCL_float_single_thread_arg_split_record(frame + 16, x, &sp, eb, n, L, frame, 1);
    CHECK("compress (split record)");
    size_t slot = 0;
    memcpy(&slot, frame + 8, sizeof slot);
    printf("split_slot %zu\n", slot);
    printf("split_stream_equal %d\n", sp == s1 && memcmp(frame + 16, a1, s1) == 0);
    printf("stream_sizes %zu %zu %zu\n", sa, sb, sh);
    return 0;
}
