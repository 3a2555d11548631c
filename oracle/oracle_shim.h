/*
 * oracle_shim.h -- lets an OpenCL C kernel written by myokit's template
 * myokit/_sim/openclsim.cl compile as plain C99 for the CPU oracle.
 *
 * TEST INFRASTRUCTURE: part of the CPU oracle that checks the CUDA path.
 * Nothing in the product imports or links it.
 *
 * - Address-space and kernel qualifiers become nothing.
 * - get_global_id(i) reads a thread-local work-item id set by the driver.
 * - <tgmath.h> makes exp/log/pow of a float argument single precision, as in
 *   OpenCL C, where math built-ins are overloaded on the argument type.
 * - native_* functions map to the full-precision functions.
 * - The 32/64-bit compare-and-swap used by the connection kernel's AtomicAdd
 *   (openclsim.cl:499-524) becomes a GCC atomic builtin.
 */
#ifndef ORACLE_SHIM_H
#define ORACLE_SHIM_H

#include <tgmath.h>

#define __kernel
#define __global
#define __private
#define __local
#define __constant const

extern __thread unsigned long orc_gid[2];
#define get_global_id(i) (orc_gid[(i)])

#define native_exp exp
#define native_log log
#define native_log10 log10
#define native_sqrt sqrt
#define native_sin sin
#define native_cos cos
#define native_tan tan

static inline unsigned int atomic_cmpxchg(volatile unsigned int *p,
                                          unsigned int cmp, unsigned int val)
{
    __atomic_compare_exchange_n(p, &cmp, val, 0, __ATOMIC_SEQ_CST,
                                __ATOMIC_SEQ_CST);
    return cmp;
}

static inline unsigned long atom_cmpxchg(volatile unsigned long *p,
                                         unsigned long cmp, unsigned long val)
{
    __atomic_compare_exchange_n(p, &cmp, val, 0, __ATOMIC_SEQ_CST,
                                __ATOMIC_SEQ_CST);
    return cmp;
}

/* OpenCL 'inline' functions get internal linkage in C99 */
#define inline static inline

#endif /* ORACLE_SHIM_H */
