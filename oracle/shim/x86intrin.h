/* Stand-in for <x86intrin.h> so the reference headers also compile on
 * aarch64 hosts.  Only __rdtsc is referenced (by the pacing code, which the
 * oracle never calls). */
#ifndef ORACLE_SHIM_X86INTRIN_H
#define ORACLE_SHIM_X86INTRIN_H
#include <stdint.h>
static inline uint64_t __rdtsc(void) { return 0; }
#endif
