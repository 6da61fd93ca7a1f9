/*
 * Test helper: the 3-D codec's float quantization and reconstruction
 * tiers (zccl_gb300/csrc/zk_szp3d.cu: sz3_quantize, sz3_value) restated in
 * C with IEEE float operations and fmaf, checked against the double steps
 * the reference takes, (int)floor((double)x * inv + 0.5) and
 * (float)((double)q * twice) (ZCCL_float.h:57-61, ZCCLd_float.c:2857).
 * Inputs: seeded random floats, floats placed on and next to the ties, and
 * quantized values of every magnitude.  Prints the mismatch count; built
 * and run by tests/test_szp3d.py with -ffp-contract=off.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    double d;
    float hi, lo;
    int ok;
} Split;

static Split split(double d)
{
    Split s;
    s.d = d;
    s.hi = (float)d;
    s.lo = (float)(d - (double)s.hi);
    s.ok = d >= 0x1p-90 && d <= 0x1p90;
    return s;
}

static float f_of(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static uint32_t u_of(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

static int32_t quant(float x, Split inv)
{
    const float t1 = fmaf(x, inv.hi, 0.5f);
    if (inv.ok && fabsf(t1) < 2048.0f) {
        const float n1 = floorf(t1), f1 = t1 - n1;
        if (f1 > 2.44140625e-4f && f1 < 0.999755859375f) return (int32_t)n1;
    }
    const float th = x * inv.hi;
    if (inv.ok && fabsf(th) < 67108864.0f) {
        const float tl = fmaf(x, inv.lo, fmaf(x, inv.hi, -th));
        const float s = th + 0.5f, bb = s - th;
        const float e = (th - (s - bb)) + (0.5f - bb);
        const float n = floorf(s);
        float fr = (s - n) + (e + tl);
        const float m = floorf(fr);
        fr = fr - m;
        if (fr > 2.44140625e-4f && fr < 0.999755859375f) return (int32_t)n + (int32_t)m;
    }
    const double v = floor((double)x * inv.d + 0.5);
    return (v >= -2147483648.0 && v < 2147483648.0) ? (int32_t)v : 0;
}

static int32_t quant_ref(float x, double inv)
{
    const double v = floor((double)x * inv + 0.5);
    return (v >= -2147483648.0 && v < 2147483648.0) ? (int32_t)v : 0;
}

static float value(int32_t q, Split tw)
{
    if (tw.ok && q == 0) return 0.0f;
    if (tw.ok && q > -16777216 && q < 16777216) {
        const float qf = (float)q, hi = qf * tw.hi;
        const float lo = fmaf(qf, tw.lo, fmaf(qf, tw.hi, -hi));
        const float r = hi + lo;
        const uint32_t rb = u_of(r) & 0x7FFFFFFFu, ex = rb >> 23;
        if (ex > 24u && ex < 254u && (rb & 0x7FFFFFu) != 0u) {
            const float half = f_of((ex - 24u) << 23), d = (hi - r) + lo;
            if (fabsf(d) < half * 0.999996185302734375f) return r;
        }
    }
    return (float)((double)q * tw.d);
}

static uint64_t st = 0x9E3779B97F4A7C15ull;
static uint64_t rnd(void)
{
    st ^= st << 13;
    st ^= st >> 7;
    st ^= st << 17;
    return st;
}

int main(int argc, char **argv)
{
    const long rounds = argc > 1 ? atol(argv[1]) : 20000;
    long bad = 0, checks = 0;
    for (long it = 0; it < rounds; it++) {
        const double eb = pow(10.0, -8.0 + 12.0 * (double)(rnd() % 1000000) / 1e6) * (1.0 + (double)(rnd() % 997) / 997.0);
        const Split inv = split(0.5 / eb), tw = split(eb * 2);
        for (int k = 0; k < 256; k++) {
            float x;
            const int mode = (int)(rnd() % 4);
            if (mode == 0) {
                x = f_of((uint32_t)rnd());
                if (isnan(x)) continue;
            } else if (mode == 1) { /* at and next to x * inv + 0.5 = j */
                const double j = (double)((int64_t)(rnd() % 200000000) - 100000000);
                x = f_of(u_of((float)((j - 0.5) / inv.d)) + (uint32_t)((int)(rnd() % 7) - 3));
            } else if (mode == 2) {
                const double j = (double)((int64_t)(rnd() % 8192) - 4096);
                x = f_of(u_of((float)((j - 0.5) / inv.d)) + (uint32_t)((int)(rnd() % 5) - 2));
            } else {
                x = (float)(((double)(rnd() % 2000001) - 1e6) * 1e-6 * (rnd() % 2 ? 1e3 : 1.0));
            }
            checks++;
            if (quant(x, inv) != quant_ref(x, inv.d)) bad++;
            const int32_t q = rnd() % 3 ? quant_ref(x, inv.d) : (int32_t)(rnd() % 33554432) - 16777216;
            checks++;
            if (u_of(value(q, tw)) != u_of((float)((double)q * tw.d))) bad++;
        }
    }
    printf("%ld %ld\n", bad, checks);
    return bad != 0;
}
