// hhp_compat.cu -- drop-ins for the reference's device-pointer launchers
// (src/include/hhp_dp_kernels.h:37-59, implemented in src/util/hhp_dp_kernels.cu:16-74).
// Same names, arguments and arithmetic meaning, so the reference's bicgstab-gpu-dp loop
// (src/entry/bicgstab_gpu_dp.c:165-196) links against libhhp_gpu.so unchanged. The vector
// operations use 128-bit loads and stores when every pointer is 16-byte aligned.
#include <cstdint>

#include "hhp_internal.h"

namespace {

__global__ void k_upd_beta(double *beta, double *rho_old, const double *rho_new, const double *alpha,
                           const double *omega) {
    // uses the old alpha/omega: they are updated later in the iteration
    *beta = (*rho_new / *rho_old) * (*alpha / *omega);
    *rho_old = *rho_new;
}
__global__ void k_upd_alpha(double *alpha, double *neg_alpha, const double *rho, const double *rv) {
    const double a = *rho / *rv;
    *alpha = a;
    *neg_alpha = -a;
}
__global__ void k_upd_omega(double *omega, double *neg_omega, const double *ts, const double *tt) {
    const double w = *ts / *tt;
    *omega = w;
    *neg_omega = -w;
}

template <bool VEC>
__global__ void k_P(double *P, const double *V, const double *R, const double *omega, const double *beta, int n) {
    const double w = *omega, b = *beta;
    const int stride = gridDim.x * blockDim.x;
    if (VEC) {
        const int n2 = n / 2;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += stride) {
            double2 p = reinterpret_cast<double2 *>(P)[i];
            const double2 v = reinterpret_cast<const double2 *>(V)[i], r = reinterpret_cast<const double2 *>(R)[i];
            p.x = (p.x - w * v.x) * b + r.x;
            p.y = (p.y - w * v.y) * b + r.y;
            reinterpret_cast<double2 *>(P)[i] = p;
        }
        if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) P[n - 1] = (P[n - 1] - w * V[n - 1]) * b + R[n - 1];
    } else {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) P[i] = (P[i] - w * V[i]) * b + R[i];
    }
}

template <bool VEC>
__global__ void k_S(double *S, const double *R, const double *V, const double *neg_alpha, int n) {
    const double na = *neg_alpha;
    const int stride = gridDim.x * blockDim.x;
    if (VEC) {
        const int n2 = n / 2;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += stride) {
            const double2 r = reinterpret_cast<const double2 *>(R)[i], v = reinterpret_cast<const double2 *>(V)[i];
            reinterpret_cast<double2 *>(S)[i] = make_double2(r.x + na * v.x, r.y + na * v.y);
        }
        if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) S[n - 1] = R[n - 1] + na * V[n - 1];
    } else {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) S[i] = R[i] + na * V[i];
    }
}

template <bool VEC>
__global__ void k_XR(double *X, double *R, const double *P, const double *S, const double *T, const double *alpha,
                     const double *omega, const double *neg_omega, int n) {
    const double a = *alpha, w = *omega, nw = *neg_omega;
    const int stride = gridDim.x * blockDim.x;
    if (VEC) {
        const int n2 = n / 2;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += stride) {
            double2 x = reinterpret_cast<double2 *>(X)[i];
            const double2 p = reinterpret_cast<const double2 *>(P)[i], s = reinterpret_cast<const double2 *>(S)[i],
                          t = reinterpret_cast<const double2 *>(T)[i];
            x.x += a * p.x + w * s.x;
            x.y += a * p.y + w * s.y;
            reinterpret_cast<double2 *>(X)[i] = x;
            reinterpret_cast<double2 *>(R)[i] = make_double2(s.x + nw * t.x, s.y + nw * t.y);
        }
        if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
            const int i = n - 1;
            X[i] += a * P[i] + w * S[i];
            R[i] = S[i] + nw * T[i];
        }
    } else {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
            X[i] += a * P[i] + w * S[i];
            R[i] = S[i] + nw * T[i];
        }
    }
}

inline bool a16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }
inline int grid_of(int n) {
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long want = (n + 511LL) / 512;
    return want < 1 ? 1 : static_cast<int>(want < 4LL * sms ? want : 4LL * sms);
}

}  // namespace

extern "C" {

void hhp_dp_vecop_P(double *P, const double *V, const double *R, const double *omega, const double *beta, int n,
                    void *s) {
    if (n <= 0) return;
    cudaStream_t st = static_cast<cudaStream_t>(s);
    if (a16(P) && a16(V) && a16(R)) k_P<true><<<grid_of(n / 2 + 1), 256, 0, st>>>(P, V, R, omega, beta, n);
    else k_P<false><<<grid_of(n), 256, 0, st>>>(P, V, R, omega, beta, n);
}

void hhp_dp_vecop_S(double *S, const double *R, const double *V, const double *neg_alpha, int n, void *s) {
    if (n <= 0) return;
    cudaStream_t st = static_cast<cudaStream_t>(s);
    if (a16(S) && a16(R) && a16(V)) k_S<true><<<grid_of(n / 2 + 1), 256, 0, st>>>(S, R, V, neg_alpha, n);
    else k_S<false><<<grid_of(n), 256, 0, st>>>(S, R, V, neg_alpha, n);
}

void hhp_dp_vecop_XR(double *X, double *R, const double *P, const double *S, const double *T, const double *alpha,
                     const double *omega, const double *neg_omega, int n, void *s) {
    if (n <= 0) return;
    cudaStream_t st = static_cast<cudaStream_t>(s);
    if (a16(X) && a16(R) && a16(P) && a16(S) && a16(T))
        k_XR<true><<<grid_of(n / 2 + 1), 256, 0, st>>>(X, R, P, S, T, alpha, omega, neg_omega, n);
    else
        k_XR<false><<<grid_of(n), 256, 0, st>>>(X, R, P, S, T, alpha, omega, neg_omega, n);
}

void hhp_dp_update_beta(double *beta, double *rho_old, const double *rho_new, const double *alpha,
                        const double *omega, void *s) {
    k_upd_beta<<<1, 1, 0, static_cast<cudaStream_t>(s)>>>(beta, rho_old, rho_new, alpha, omega);
}

void hhp_dp_update_alpha(double *alpha, double *neg_alpha, const double *rho, const double *rv, void *s) {
    k_upd_alpha<<<1, 1, 0, static_cast<cudaStream_t>(s)>>>(alpha, neg_alpha, rho, rv);
}

void hhp_dp_update_omega(double *omega, double *neg_omega, const double *ts, const double *tt, void *s) {
    k_upd_omega<<<1, 1, 0, static_cast<cudaStream_t>(s)>>>(omega, neg_omega, ts, tt);
}

}  // extern "C"
