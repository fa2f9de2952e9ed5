// exp(x) computed by the same operations in the same order on the host and on the device, so that
// both give the same bits: the batched HMC turns its parameters x = ln C_l into C_l with it both in
// the device-resident leapfrog (k_hmc.cu) and in the host-driven one (cg_hmc.cpp), whose chains
// therefore agree exactly.
//
// Method: Cody and Waite's argument reduction, x = n ln2 + r with n = rint(x / ln2) and ln 2 split
// into a 32-bit head (n * head exact for |n| < 2^21) and a tail, then e^r, |r| <= ln2 / 2, by its
// Taylor series to degree 13 (the first omitted term is below 4e-18 relative) in Horner form, and
// the scaling by 2^n.  Every product and sum is rounded separately (no fused multiply-add; the host
// side is compiled with -ffp-contract=off).  Error: a few ulp; exp(x) overflows to +inf above 709.78
// and flushes to 0 below -745.
#pragma once

#include <cmath>

namespace cg {

#ifdef __CUDA_ARCH__
#define CG_EXP_MUL(a, b) __dmul_rn((a), (b))
#define CG_EXP_ADD(a, b) __dadd_rn((a), (b))
#define CG_EXP_SUB(a, b) __dsub_rn((a), (b))
#else
#define CG_EXP_MUL(a, b) ((a) * (b))
#define CG_EXP_ADD(a, b) ((a) + (b))
#define CG_EXP_SUB(a, b) ((a) - (b))
#endif

#ifdef __CUDACC__
__host__ __device__
#endif
inline double exp_same(double x)
{
    if (x != x) return x;
    if (x > 709.78) return INFINITY;
    if (x < -745.2) return 0.0;
    const double ln2_hi = 0x1.62e42ffp-1;               // ln 2 to 32 bits
    const double ln2_lo = -0x1.718432a1b0e26p-35;       // ln 2 - ln2_hi
    const double inv_ln2 = 0x1.71547652b82fep+0;        // 1 / ln 2
    const double c[14] = {1.0, 1.0, 0.5, 1.0 / 6, 1.0 / 24, 1.0 / 120, 1.0 / 720, 1.0 / 5040, 1.0 / 40320,
                          1.0 / 362880, 1.0 / 3628800, 1.0 / 39916800, 1.0 / 479001600, 1.0 / 6227020800.0};
    const double n = rint(CG_EXP_MUL(x, inv_ln2));
    const double r = CG_EXP_SUB(CG_EXP_SUB(x, CG_EXP_MUL(n, ln2_hi)), CG_EXP_MUL(n, ln2_lo));
    double s = c[13];
    for (int k = 12; k >= 0; --k) s = CG_EXP_ADD(CG_EXP_MUL(s, r), c[k]);
    return ldexp(s, (int)n);
}

#undef CG_EXP_MUL
#undef CG_EXP_ADD
#undef CG_EXP_SUB

}  // namespace cg
