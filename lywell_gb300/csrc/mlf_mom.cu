// Dense method-of-moments operator on the GPU (modMoM.f90:85-128 fill,
// MatxVec_MoM modMoM.f90:273-277): the full N x N impedance matrix in FP64,
// filled on the device by the same Z_mn element as the near field, and a
// matvec that streams it once per group of four right-hand sides.  A
// context made with MLF_FLAG_DENSE_MOM holds this operator instead of the
// octree; CGS, excitation and RCS run on it unchanged.  At N = 30720 the
// matrix is 15 GB, within HBM, so it also serves as the exact reference for
// the MLFMA matvec error.
#include <cuda_runtime.h>

#include <algorithm>

#include "mlf_internal.h"
#include "mlf_zmn.cuh"

namespace mlf {

#define CK(call)                                             \
    do {                                                     \
        if (!cuda_ok(c, (call), #call)) return MLF_E_CUDA;   \
    } while (0)

// row m per block: Z[m][n] for all n (row-major)
__global__ void k_mom_fill(int N, const double* __restrict__ t_baric, const double* __restrict__ t_baric_sub,
                           const double* __restrict__ p_coord, const int* __restrict__ e_t, const int* __restrict__ e_po,
                           const double* __restrict__ e_long, double w, double w_smue, double c72,
                           double2* __restrict__ Z) {
    const int m = blockIdx.x;
    for (int n = threadIdx.x; n < N; n += blockDim.x)
        Z[(size_t)m * N + n] = zmn_mom(m, n, t_baric, t_baric_sub, p_coord, e_t, e_po, e_long, w, w_smue, c72);
}

// y(m, c) = sum_n Z[m][n] x(n, c): one warp per row, four columns per pass
__global__ void k_mom_gemv(int N, int nrhs, int ld, const double2* __restrict__ Z, const double2* __restrict__ x,
                           double2* __restrict__ y) {
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (gw >= N) return;
    const int m = (int)gw;
    const double2* zr = Z + (size_t)m * N;
    for (int c0 = 0; c0 < nrhs; c0 += 4) {
        double ar[4] = {0, 0, 0, 0}, ai[4] = {0, 0, 0, 0};
        for (int n = lane; n < N; n += 32) {
            const double2 z = zr[n];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (c0 + u < nrhs) {
                    const double2 v = x[(size_t)(c0 + u) * ld + n];
                    ar[u] = fma(z.x, v.x, ar[u]); ar[u] = fma(-z.y, v.y, ar[u]);
                    ai[u] = fma(z.x, v.y, ai[u]); ai[u] = fma(z.y, v.x, ai[u]);
                }
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                ar[u] += __shfl_xor_sync(0xffffffff, ar[u], o);
                ai[u] += __shfl_xor_sync(0xffffffff, ai[u], o);
            }
        }
        if (lane == 0)
            for (int u = 0; u < 4 && c0 + u < nrhs; ++u) y[(size_t)(c0 + u) * ld + m] = make_double2(ar[u], ai[u]);
    }
}

int dense_setup(Ctx* c) {
    CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    for (int i = 0; i < 8; ++i) CK(cudaEventCreate(&c->ev[i]));
    int st;
    if ((st = upload_geometry(c))) return st;
    const size_t bytes = (size_t)c->N * c->N * sizeof(double2);
    size_t fre = 0, tot = 0;
    CK(cudaMemGetInfo(&fre, &tot));
    if (bytes + ((size_t)1 << 30) > fre) {
        c->err = "dense MoM matrix does not fit in device memory";
        return MLF_E_NOMEM;
    }
    CK(cudaMalloc(&c->dZdense, bytes));
    const double c72 = (double)(1.0f / 72.0f);   // (1./72.) in single precision, as the near field
    k_mom_fill<<<c->N, 256, 0, c->stream>>>(c->N, c->dt_baric, c->dt_baric_sub, c->dp_coord, c->de_t, c->de_po,
                                            c->de_long, c->ph.w, c->ph.w * c->ph.smue, c72, c->dZdense);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->stream));
    return MLF_OK;
}

int dense_matvec(Ctx* c, const double2* x, double2* y, int nrhs, int ld, cudaStream_t s) {
    const long long threads = (long long)c->N * 32;
    k_mom_gemv<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(c->N, nrhs, ld, c->dZdense, x, y);
    return cuda_ok(c, cudaGetLastError(), "dense matvec") ? MLF_OK : MLF_E_CUDA;
}

}  // namespace mlf
