// Reverso two-reservoir magma model (Reverso et al. 2014): predicted GPS
// displacements, residuals and the diagonal-Cd data log-likelihood of a batch
// of samples, in FP64.
//
// Reference: models/reverso/lib/libreverso/reverso.cc:37-142 (the forward model
// the default strategy calls, Source.cc:56-88), Source.cc:92-123 (residuals) and
// Fast.py:52-90 (llk = norm - |L r|²/2, L = chol(Cd⁻¹), per sample on the host).
// The reference's algebra is kept, quirks included: τ uses H_c^γ_s
// (reverso.cc:60-61) and the pressures 1 - exp(-t/τ) (reverso.cc:79).  The E/N
// split u_r·(cos φ, sin φ) with φ = atan2(y, x) is evaluated as (x, y)·F with
// u_r = r F, which is the same quantity without the angle (and is 0 at r = 0,
// where the reference's atan2(0, 0) = 0 also gives 0).
//
// Work decomposition: one warp per sample (grid-stride), lanes over observation
// points; per-sample constants are computed by every lane; each lane sums its
// points' w·r² in a fixed order and the warp reduces in a fixed butterfly, so
// results do not depend on the launch.
#include <math.h>
#include <stdint.h>

#include "common.cuh"
#include "internal.h"

namespace ag {

constexpr int kRevWarps = 8;

__global__ void __launch_bounds__(kRevWarps * 32)
reverso_llk_kernel(ag_reverso_model M, const double* __restrict__ theta, int n, double norm,
                   const uint32_t* __restrict__ mask, double* __restrict__ llk,
                   double* __restrict__ predicted) {
    const double PI = 3.14159265358979323846;
    const int lane = threadIdx.x & 31;
    const int stride = gridDim.x * kRevWarps;
    for (int i = blockIdx.x * kRevWarps + (threadIdx.x >> 5); i < n; i += stride) {
        if (mask && mask[i]) continue;
        const double* th = theta + (size_t)i * M.nparams;
        const double Qin = th[M.qin_idx], H_s = th[M.hs_idx], H_d = th[M.hd_idx];
        const double a_s = th[M.as_idx], a_d = th[M.ad_idx], a_c = th[M.ac_idx];
        const double v = M.v, G = M.G;
        // reservoir constants (reverso.cc:44-68)
        const double q = a_d / a_s;
        const double k = q * q * q;
        const double H_c = H_d - H_s;
        const double gamma_s = 8.0 * (1.0 - v) / (3.0 * PI);
        const double gamma_d = gamma_s;
        const double gamma_r = gamma_s + gamma_d * k;
        const double as3 = a_s * a_s * a_s, ad3 = a_d * a_d * a_d, ac4 = a_c * a_c * a_c * a_c;
        const double tau = (8.0 * M.mu * pow(H_c, gamma_s) * gamma_d * k * as3) / (G * ac4 * gamma_r);
        const double A = gamma_d * k / gamma_r *
                         (M.drho * M.g * H_c - 8.0 * gamma_s * M.mu * Qin * H_c / (PI * ac4 * gamma_r));
        const double c1 = G * Qin / (PI * as3 * gamma_r);
        const double cd = gamma_s / (gamma_d * k);
        const double H2_s = H_s * H_s, H2_d = H_d * H_d;
        const double ks = as3 * (1.0 - v) / G, kd = ad3 * (1.0 - v) / G;
        double acc = 0.0;
        for (int j = lane; j < M.n_obs; j += 32) {
            const double t = M.txy[3 * j], x = M.txy[3 * j + 1], y = M.txy[3 * j + 2];
            // pressures (reverso.cc:78-83)
            const double f0 = A * (1.0 - exp(-t / tau));
            const double f1 = c1 * t;
            const double dP_s = f1 + f0;
            const double dP_d = f1 - f0 * cd;
            // Green's functions of the two reservoirs (reverso.cc:109-142)
            const double r2 = x * x + y * y;
            const double R2_s = r2 + H2_s, R2_d = r2 + H2_d;
            const double alpha_s = (gamma_s == 1.0) ? 1.0 : 4.0 * H2_s / (PI * R2_s);
            const double alpha_d = (gamma_d == 1.0) ? 1.0 : 4.0 * H2_d / (PI * R2_d);
            const double f_s = ks * alpha_s / (R2_s * sqrt(R2_s));
            const double f_d = kd * alpha_d / (R2_d * sqrt(R2_d));
            const double F = f_s * dP_s + f_d * dP_d;            // u_r / r
            const double uz = H_s * f_s * dP_s + H_d * f_d * dP_d;
            const double ue = M.east_cos ? x * F : y * F;
            const double un = M.east_cos ? y * F : x * F;
            if (predicted) {
                double* out = predicted + (size_t)i * 3 * M.n_obs + 3 * j;
                out[0] = ue;
                out[1] = un;
                out[2] = uz;
            }
            const double* d = M.d + 3 * j;
            const double* w = M.w + 3 * j;
            const double re = ue - d[0], rn = un - d[1], rz = uz - d[2];
            acc += w[0] * re * re + w[1] * rn * rn + w[2] * rz * rz;
        }
        acc = warp_sum(acc);
        if (lane == 0) llk[i] = norm - 0.5 * acc;
    }
}

}  // namespace ag

using namespace ag;

extern "C" int ag_reverso_llk(const ag_reverso_model* model, const double* theta, int32_t n, double norm,
                              const uint32_t* mask, double* llk, double* predicted, void* stream) {
    AG_REQUIRE(model != nullptr && theta != nullptr && llk != nullptr, "null argument");
    AG_REQUIRE(n > 0, "n must be positive (got %d)", n);
    const ag_reverso_model M = *model;
    AG_REQUIRE(M.txy && M.d && M.w && M.n_obs > 0, "observation arrays must be given (n_obs=%d)", M.n_obs);
    const int idx[6] = {M.qin_idx, M.hs_idx, M.hd_idx, M.as_idx, M.ad_idx, M.ac_idx};
    for (int k = 0; k < 6; ++k)
        AG_REQUIRE(idx[k] >= 0 && idx[k] < M.nparams, "parameter index %d out of range [0, %d)", idx[k],
                   M.nparams);
    AG_REQUIRE(M.G > 0.0, "shear modulus must be positive");
    int dev = 0, sms = 0;
    int rc = cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
    if (rc) return rc;
    rc = cuda_status(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "multiProcessorCount");
    if (rc) return rc;
    const int grid = min((n + kRevWarps - 1) / kRevWarps, 8 * sms);
    reverso_llk_kernel<<<grid, kRevWarps * 32, 0, as_stream(stream)>>>(M, theta, n, norm, mask, llk, predicted);
    return launch_status("reverso_llk_kernel");
}
