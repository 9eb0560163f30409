// Accuracy probes of the library's own arithmetic (bm_scalar.h) on the
// device, each beside CUDA's function of the same argument, so that tests can
// measure both against float64 references and CUDA's documented error
// bounds.  The substep kernels call the bm_* forms (the same IEEE operation
// sequence as the oracle); these probes are not on the substep path.
#include "bm_device.cuh"
#include "bm_internal.h"

namespace bm {

__global__ void k_math_probe_f(int kind, const float* __restrict__ x, int n, float* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float v = x[i];
    float ours, cuda;
    if (kind == 0) {
        ours = bm_logf(v);
        cuda = logf(v);
    } else if (kind == 1) {
        ours = bm_expf(v);
        cuda = expf(v);
    } else {
        ours = bm_expm1f(v);
        cuda = expm1f(v);
    }
    out[2 * i] = ours;
    out[2 * i + 1] = cuda;
}

__global__ void k_math_probe_d(int kind, const double* __restrict__ x, const double* __restrict__ y, int n,
                               double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double ours, cuda;
    if (kind == 2) {
        ours = bm_atan2(y[i], x[i]);
        cuda = atan2(y[i], x[i]);
    } else {
        double s, c;
        bm_sincos(x[i], &s, &c);
        ours = kind == 0 ? s : c;
        cuda = kind == 0 ? sin(x[i]) : cos(x[i]);
    }
    out[2 * i] = ours;
    out[2 * i + 1] = cuda;
}

// Row-major 3x3 matrices in, U, sigma, V (bm_svd3) and R (bm_polar3) out.
__global__ void k_svd_probe(const float* __restrict__ A, int n, float* U, float* sigma, float* V, float* R) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    bm_m33 a;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) a.m[r][c] = A[9 * i + 3 * r + c];
    bm_m33 u, v;
    bm_v3 s;
    bm_svd3(a, &u, &s, &v);
    const bm_m33 rot = bm_polar3(a);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            U[9 * i + 3 * r + c] = u.m[r][c];
            V[9 * i + 3 * r + c] = v.m[r][c];
            R[9 * i + 3 * r + c] = rot.m[r][c];
        }
    sigma[3 * i] = s.x;
    sigma[3 * i + 1] = s.y;
    sigma[3 * i + 2] = s.z;
}

}  // namespace bm

extern "C" {

int bm_math_probe_f(int kind, const float* x, int n, float* out, void* stream) {
    if (kind < 0 || kind > 2 || n < 0 || (n > 0 && (!x || !out))) return bm::fail(BM_ERR_ARGUMENT, "invalid arguments");
    if (n == 0) return BM_OK;
    bm::k_math_probe_f<<<bm::grid_for(n), bm::kBlock, 0, reinterpret_cast<cudaStream_t>(stream)>>>(kind, x, n, out);
    return bm::check_cuda("math_probe_f");
}

int bm_math_probe_d(int kind, const double* x, const double* y, int n, double* out, void* stream) {
    if (kind < 0 || kind > 2 || n < 0 || (n > 0 && (!x || !out || (kind == 2 && !y))))
        return bm::fail(BM_ERR_ARGUMENT, "invalid arguments");
    if (n == 0) return BM_OK;
    bm::k_math_probe_d<<<bm::grid_for(n), bm::kBlock, 0, reinterpret_cast<cudaStream_t>(stream)>>>(kind, x, y, n, out);
    return bm::check_cuda("math_probe_d");
}

int bm_svd_probe(const float* A, int n, float* U, float* sigma, float* V, float* R, void* stream) {
    if (n < 0 || (n > 0 && (!A || !U || !sigma || !V || !R))) return bm::fail(BM_ERR_ARGUMENT, "invalid arguments");
    if (n == 0) return BM_OK;
    bm::k_svd_probe<<<bm::grid_for(n), bm::kBlock, 0, reinterpret_cast<cudaStream_t>(stream)>>>(A, n, U, sigma, V, R);
    return bm::check_cuda("svd_probe");
}

}  // extern "C"
