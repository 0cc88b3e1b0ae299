// sph_kernel.cuh -- the smoothing kernel W(r) and its gradient factor, shared
// by the pair operators (pairs.cu) and the salinity flux (scalar.cu).
#pragma once

#include "bsc_internal.cuh"

namespace bsc {

// ---- smoothing kernel --------------------------------------------------------
// grad_i W = F(r) (x_i - x_j).  Hybrid (kernel.f90:94-162):
//   r <  h: F = A (9r/h^3 - 12/h^2) + B (3r/h^3 - 6/(r h))
//   r >= h: F = -(A + B) (3/(r h)) (2 - r/h)^2
// with A = 0.1*10/(28*3.14 h^2), B = 0.9/(3*3.14 h^2) (3.14 is the
// reference's single-precision literal).  Wendland C2 (kernel.f90:102-103):
//   F = -35/(4*3.14 h^4) (1 - r/(2h))^3.
template <typename R>
__device__ __forceinline__ R grad_factor(const KParams& K, R r) {
    if (K.kernel == BSC_KERNEL_WENDLAND_C2) {
        // a = 1 - r/(2h) in one FMA; -F a^3 as (-F a) a^2: four operations
        const R a = fma(-r, (R)K.half_inv_h, (R)1);
        return (-(R)K.wend_F * a) * (a * a);
    }
    const R q = r * (R)K.inv_h;
    // A (9r/h^3 - 12/h^2) + B (3r/h^3 - 6/(rh)) = (9A+3B) r/h^3 - 12A/h^2 - 6B/(rh)
    const R inv_rh = (R)K.inv_h / r;
    if (q < (R)1) return (R)K.hyb_n1 * r - (R)K.hyb_n0 - (R)K.hyb_n2 * inv_rh;
    R a = (R)2 - q;
    return -(R)K.hyb_f * inv_rh * (a * a);
}

// W(r) (kernel.f90:34-66 and the Wendland comment at :42-43)
template <typename R>
__device__ __forceinline__ R kern_w(const KParams& K, R r) {
    const R q = r * (R)K.inv_h;
    if (K.kernel == BSC_KERNEL_WENDLAND_C2) {
        R a = (R)1 - (R)0.5 * q, a2 = a * a;
        return (R)K.wend_W * ((R)1 + (R)2 * q) * (a2 * a2);
    }
    const R A = (R)K.hyb_A, B = (R)K.hyb_B;
    if (q < (R)1) return A * ((R)4 - (R)6 * q * q + (R)3 * q * q * q) + B * (q * q * q - (R)6 * q + (R)6);
    R a = (R)2 - q;
    return (A + B) * (a * a * a);
}

}  // namespace bsc
