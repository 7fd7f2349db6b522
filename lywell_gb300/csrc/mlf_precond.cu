// Neighbourhood-inverse preconditioner (an addition of this library; the
// reference offers ILU0/ILUT, modIterativo.f90:1805-1976, 2432-2883).
//
// For each leaf box b with neighbourhood S (the sorted near list of b, i.e.
// the column set of every row of b in the near-field CSR) take
// A = Znear[S, S] (entries absent from the CSR are zero) and keep the rows of
// A^-1 that belong to b's own bases.  Stacked, these rows form M with the
// near CSR's own sparsity pattern; M is fixed and linear, so
// right-preconditioned CGS stays valid.  Rows of A^-1 solve A^T X = E_own.
//
// Set-up: one CTA per box, Gaussian elimination with partial pivoting
// (largest |a|^2, first row on ties) in FP64 on a per-CTA workspace slab, for
// neighbourhoods of up to NBI_FP64_MAX unknowns; larger ones go to the
// blocked FP32 LU of mlf_nbhd_lu.cu (mlf_set_nearinv_precision overrides).
// Apply: a warp-per-row SpMV with the near CSR pattern.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "mlf_internal.h"

namespace mlf {

#define CK(call)                                             \
    do {                                                     \
        if (!cuda_ok(c, (call), #call)) return MLF_E_CUDA;   \
    } while (0)

__device__ __forceinline__ int bsearch_sorted(const int* S, int n, int v) {
    int lo = 0, hi = n - 1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        const int s = S[mid];
        if (s == v) return mid;
        if (s < v) lo = mid + 1;
        else hi = mid - 1;
    }
    return -1;
}

__device__ __forceinline__ double2 zdiv(double2 a, double2 b) {
    const double d = b.x * b.x + b.y * b.y;
    return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}

constexpr int NBI_THREADS = 256;
// neighbourhoods of more unknowns go to the blocked FP32 LU unless FP64 is asked for
constexpr int NBI_FP64_MAX = 768;

__global__ void __launch_bounds__(NBI_THREADS)
k_nbhd_inverse(int b0, int nb, const int* __restrict__ box_ptr, const int* __restrict__ box_bases,
               const int* __restrict__ own_sorted, int own_only, const int* __restrict__ ia,
               const int* __restrict__ ja, const float2* __restrict__ Z, size_t slab, double2* __restrict__ work,
               double2* __restrict__ M, const long long* __restrict__ boff, int* __restrict__ bad) {
    const int b = b0 + blockIdx.x;
    if (b >= nb) return;
    const int tid = threadIdx.x, bd = blockDim.x;
    const int m0 = box_bases[box_ptr[b]];
    const int nown = box_ptr[b + 1] - box_ptr[b];
    // neighbourhood S: the box's near list, or (own_only) its own bases, sorted
    const int n = own_only ? nown : ia[m0 + 1] - ia[m0];
    const int* S = own_only ? own_sorted + box_ptr[b] : ja + ia[m0];
    double2* At = work + (size_t)blockIdx.x * slab;   // n x n, row-major, holds A^T
    double2* X = At + (size_t)n * n;                   // n x nown
    for (int i = tid; i < n * n; i += bd) At[i] = make_double2(0, 0);
    for (int i = tid; i < n * nown; i += bd) X[i] = make_double2(0, 0);
    __syncthreads();
    for (int r = tid; r < n; r += bd) {
        const int m = S[r];
        for (int q = ia[m]; q < ia[m + 1]; ++q) {
            const int pos = bsearch_sorted(S, n, ja[q]);
            if (pos >= 0) At[(size_t)pos * n + r] = make_double2((double)Z[q].x, (double)Z[q].y);
        }
    }
    for (int i = tid; i < nown; i += bd) {
        const int pos = bsearch_sorted(S, n, box_bases[box_ptr[b] + i]);
        X[(size_t)pos * nown + i] = make_double2(1.0, 0.0);
    }
    __shared__ double s_val[NBI_THREADS / 32];
    __shared__ int s_idx[NBI_THREADS / 32];
    __shared__ int s_piv;
    __shared__ int s_sing;
    if (tid == 0) s_sing = 0;
    __syncthreads();
    for (int k = 0; k < n; ++k) {
        // pivot: largest |a|^2 in column k at or below the diagonal, first on ties
        double best = -1.0;
        int bi = n;
        for (int i = k + tid; i < n; i += bd) {
            const double2 a = At[(size_t)i * n + k];
            const double v = a.x * a.x + a.y * a.y;
            if (v > best) { best = v; bi = i; }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const double ov = __shfl_xor_sync(0xffffffff, best, o);
            const int oi = __shfl_xor_sync(0xffffffff, bi, o);
            if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
        }
        if ((tid & 31) == 0) { s_val[tid >> 5] = best; s_idx[tid >> 5] = bi; }
        __syncthreads();
        if (tid == 0) {
            double bv = s_val[0];
            int bx = s_idx[0];
            for (int w = 1; w < bd / 32; ++w)
                if (s_val[w] > bv || (s_val[w] == bv && s_idx[w] < bx)) { bv = s_val[w]; bx = s_idx[w]; }
            s_piv = bx;
            if (!(bv > 0.0)) s_sing = 1;
        }
        __syncthreads();
        if (s_sing) break;
        const int piv = s_piv;
        if (piv != k) {
            for (int j = tid; j < n; j += bd) {
                const double2 t = At[(size_t)k * n + j];
                At[(size_t)k * n + j] = At[(size_t)piv * n + j];
                At[(size_t)piv * n + j] = t;
            }
            for (int j = tid; j < nown; j += bd) {
                const double2 t = X[(size_t)k * nown + j];
                X[(size_t)k * nown + j] = X[(size_t)piv * nown + j];
                X[(size_t)piv * nown + j] = t;
            }
        }
        __syncthreads();
        const double2 d = At[(size_t)k * n + k];
        for (int i = k + 1 + tid; i < n; i += bd) At[(size_t)i * n + k] = zdiv(At[(size_t)i * n + k], d);
        __syncthreads();
        const int rows = n - k - 1, wcols = (n - k - 1) + nown;
        for (int e = tid; e < rows * wcols; e += bd) {
            const int i = k + 1 + e / wcols, jj = e % wcols;
            const double2 f = At[(size_t)i * n + k];
            double2* dst;
            double2 src;
            if (jj < n - k - 1) {
                dst = &At[(size_t)i * n + k + 1 + jj];
                src = At[(size_t)k * n + k + 1 + jj];
            } else {
                dst = &X[(size_t)i * nown + (jj - (n - k - 1))];
                src = X[(size_t)k * nown + (jj - (n - k - 1))];
            }
            double2 v = *dst;
            v.x -= f.x * src.x - f.y * src.y;
            v.y -= f.x * src.y + f.y * src.x;
            *dst = v;
        }
        __syncthreads();
    }
    if (s_sing) {
        if (tid == 0) atomicMin(bad, b + 1);
        return;
    }
    for (int k = n - 1; k >= 0; --k) {
        const double2 d = At[(size_t)k * n + k];
        for (int j = tid; j < nown; j += bd) X[(size_t)k * nown + j] = zdiv(X[(size_t)k * nown + j], d);
        __syncthreads();
        for (int e = tid; e < k * nown; e += bd) {
            const int i = e / nown, j = e % nown;
            const double2 f = At[(size_t)i * n + k];
            const double2 s = X[(size_t)k * nown + j];
            double2 v = X[(size_t)i * nown + j];
            v.x -= f.x * s.x - f.y * s.y;
            v.y -= f.x * s.y + f.y * s.x;
            X[(size_t)i * nown + j] = v;
        }
        __syncthreads();
    }
    if (!own_only) {
        for (int e = tid; e < nown * n; e += bd) {
            const int i = e / n, j = e % n;
            const int g = box_bases[box_ptr[b] + i];
            M[(size_t)ia[g] + j] = X[(size_t)j * nown + i];
        }
    } else {
        // compact block: row i of the own-box inverse at boff[b] + i*nown
        for (int e = tid; e < nown * nown; e += bd) {
            const int i = e / nown, j = e % nown;
            M[boff[b] + e] = X[(size_t)j * nown + i];
        }
    }
}

// y[:, col] = blockdiag(M_b) x[:, col]; warp per (box-sorted row p, column)
__global__ void k_blockdiag_apply(int N, int nrhs, const int* __restrict__ box_ptr,
                                  const int* __restrict__ box_of_sorted, const int* __restrict__ perm,
                                  const long long* __restrict__ boff, const double2* __restrict__ M,
                                  const double2* __restrict__ x, double2* __restrict__ y) {
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (gw >= N * nrhs) return;
    const int p = gw % N, col = gw / N;
    const int b = box_of_sorted[p], j0 = box_ptr[b], n = box_ptr[b + 1] - j0, i = p - j0;
    const double2* row = M + boff[b] + (size_t)i * n;
    const double2* xc = x + (size_t)col * N;
    double sr = 0, si = 0;
    for (int j = lane; j < n; j += 32) {
        const double2 a = row[j], v = xc[perm[j0 + j]];
        sr = fma(a.x, v.x, sr); sr = fma(-a.y, v.y, sr);
        si = fma(a.x, v.y, si); si = fma(a.y, v.x, si);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sr += __shfl_xor_sync(0xffffffff, sr, o);
        si += __shfl_xor_sync(0xffffffff, si, o);
    }
    if (lane == 0) y[(size_t)col * N + perm[p]] = make_double2(sr, si);
}

// y[:, col] = M x[:, col], one warp per (row, column), near CSR pattern
__global__ void k_spmv_z(int N, int nrhs, const int* __restrict__ ia, const int* __restrict__ ja,
                         const double2* __restrict__ M, const double2* __restrict__ x, double2* __restrict__ y) {
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (gw >= N * nrhs) return;
    const int m = gw % N, col = gw / N;
    const double2* xc = x + (size_t)col * N;
    double sr = 0, si = 0;
    for (int q = ia[m] + lane; q < ia[m + 1]; q += 32) {
        const double2 a = M[q], v = xc[ja[q]];
        sr = fma(a.x, v.x, sr); sr = fma(-a.y, v.y, sr);
        si = fma(a.x, v.y, si); si = fma(a.y, v.x, si);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sr += __shfl_xor_sync(0xffffffff, sr, o);
        si += __shfl_xor_sync(0xffffffff, si, o);
    }
    if (lane == 0) y[(size_t)col * N + m] = make_double2(sr, si);
}

// FP32 copies of the same operator, for the FP32 inner solves of mlf_solve mode 1
__global__ void k32_blockdiag_apply(int N, int nrhs, const int* __restrict__ box_ptr,
                                    const int* __restrict__ box_of_sorted, const int* __restrict__ perm,
                                    const long long* __restrict__ boff, const float2* __restrict__ M,
                                    const float2* __restrict__ x, float2* __restrict__ y) {
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (gw >= N * nrhs) return;
    const int p = gw % N, col = gw / N;
    const int b = box_of_sorted[p], j0 = box_ptr[b], n = box_ptr[b + 1] - j0, i = p - j0;
    const float2* row = M + boff[b] + (size_t)i * n;
    const float2* xc = x + (size_t)col * N;
    float sr = 0.f, si = 0.f;
    for (int j = lane; j < n; j += 32) {
        const float2 a = row[j], v = xc[perm[j0 + j]];
        sr = fmaf(a.x, v.x, sr); sr = fmaf(-a.y, v.y, sr);
        si = fmaf(a.x, v.y, si); si = fmaf(a.y, v.x, si);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sr += __shfl_xor_sync(0xffffffff, sr, o);
        si += __shfl_xor_sync(0xffffffff, si, o);
    }
    if (lane == 0) y[(size_t)col * N + perm[p]] = make_float2(sr, si);
}

__global__ void k32_spmv_z(int N, int nrhs, const int* __restrict__ ia, const int* __restrict__ ja,
                           const float2* __restrict__ M, const float2* __restrict__ x, float2* __restrict__ y) {
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (gw >= N * nrhs) return;
    const int m = gw % N, col = gw / N;
    const float2* xc = x + (size_t)col * N;
    float sr = 0.f, si = 0.f;
    for (int q = ia[m] + lane; q < ia[m + 1]; q += 32) {
        const float2 a = M[q], v = xc[ja[q]];
        sr = fmaf(a.x, v.x, sr); sr = fmaf(-a.y, v.y, sr);
        si = fmaf(a.x, v.y, si); si = fmaf(a.y, v.x, si);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sr += __shfl_xor_sync(0xffffffff, sr, o);
        si += __shfl_xor_sync(0xffffffff, si, o);
    }
    if (lane == 0) y[(size_t)col * N + m] = make_float2(sr, si);
}

__global__ void k_d2f(size_t n, const double2* __restrict__ a, float2* __restrict__ b) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        b[i] = make_float2((float)a[i].x, (float)a[i].y);
}

int device_nearinv_apply32(Ctx* c, const float2* y, float2* x, int nrhs, cudaStream_t s) {
    if (!c->nearinv_ok) {
        c->err = "neighbourhood-inverse preconditioner not built";
        return MLF_E_STATE;
    }
    if (!c->dMinv32) {
        CK(cudaMalloc(&c->dMinv32, std::max<long long>(c->minv_len, 1) * sizeof(float2)));
        k_d2f<<<4096, 256, 0, s>>>((size_t)c->minv_len, c->dMinv, c->dMinv32);
    }
    const long long warps = (long long)c->N * nrhs;
    if (c->nearinv_own && nrhs > 1) {
        // blocks of columns: per-box GEMMs on a box-sorted copy of y
        const size_t need = (size_t)c->N * nrhs;
        if (c->pre_xs_cap < need) {
            if (c->dpre_xs) cudaFree(c->dpre_xs);
            c->dpre_xs = nullptr;
            CK(cudaMalloc(&c->dpre_xs, need * sizeof(float2)));
            c->pre_xs_cap = need;
        }
        int st;
        if ((st = device_blk_pack(c, nullptr, y, c->N, nrhs, c->dpre_xs, s))) return st;
        if (warp_engine(blk_engine_of(c))) return device_own_warp32(c, c->dboff, c->dMinv32, c->dpre_xs, nrhs, x, s);
        return device_own_blocks32(c, c->dboff, c->dMinv32, c->dpre_xs, nrhs, x, s);
    }
    if (!c->nearinv_own && nrhs > 1) {
        // blocks of columns: the near-pattern inverse as box-pair blocks, one GEMM engine pass
        const size_t need = (size_t)c->N * nrhs;
        if (c->pre_xs_cap < need) {
            if (c->dpre_xs) cudaFree(c->dpre_xs);
            c->dpre_xs = nullptr;
            CK(cudaMalloc(&c->dpre_xs, need * sizeof(float2)));
            c->pre_xs_cap = need;
        }
        int st;
        if (warp_engine(blk_engine_of(c))) {   // one warp per basis on the CSR values
            if ((st = device_blk_pack(c, nullptr, y, c->N, nrhs, c->dpre_xs, s))) return st;
            return device_near_pattern_warp32(c, c->dMinv32, c->dpre_xs, nrhs, x, s);
        }
        if (!c->dMinvblk) {
            if ((st = device_blocks_from_csr(c, c->dMinv32, &c->dMinvblk))) return st;
            tc_drop_precond(c);
        }
        if ((st = device_blk_pack(c, nullptr, y, c->N, nrhs, c->dpre_xs, s))) return st;
        if (blk_engine_of(c) == 4) return device_near_pattern_tc(c, c->dMinvblk, c->dpre_xs, nrhs, x, s);
        return device_near_pattern_apply32(c, c->dMinvblk, c->dpre_xs, nrhs, x, s);
    }
    if (c->nearinv_own)
        k32_blockdiag_apply<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, s>>>(
            c->N, nrhs, c->dbox_ptr, c->dbox_of_sorted, c->dperm, c->dboff, c->dMinv32, y, x);
    else
        k32_spmv_z<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, s>>>(c->N, nrhs, c->dia, c->dja, c->dMinv32, y, x);
    return cuda_ok(c, cudaGetLastError(), "nearinv apply32") ? MLF_OK : MLF_E_CUDA;
}

int device_nearinv_setup(Ctx* c, int* bad_box, int own_only) {
    DevScope ds;
    if (need_tree(c)) return MLF_E_STATE;
    const int nl = c->nlev;
    const Level& leaf = c->lv[nl];
    int nmax = 0, nownmax = 0;
    for (int b = 0; b < leaf.nb; ++b) {
        nmax = std::max(nmax, c->near_ptr[b + 1] - c->near_ptr[b]);
        nownmax = std::max(nownmax, c->box_ptr[b + 1] - c->box_ptr[b]);
    }
    if (own_only) nmax = nownmax;
    const size_t slab = (size_t)nmax * nmax + (size_t)nmax * nownmax;
    int batch = (int)std::min<size_t>(leaf.nb, std::max<size_t>(1, ((size_t)1 << 30) / (slab * sizeof(double2))));
    batch = std::min(batch, 4096);
    if (c->dMinv) cudaFree(c->dMinv);
    if (c->dboff) cudaFree(c->dboff);
    if (c->dMinv32) cudaFree(c->dMinv32);
    if (c->dMinvblk) cudaFree(c->dMinvblk);
    c->dMinvblk = nullptr;
    tc_drop_precond(c);
    if (c->dMinv_base) cudaFree(c->dMinv_base);
    c->dMinv_base = nullptr;
    c->dMinv = nullptr;
    c->dboff = nullptr;
    c->dMinv32 = nullptr;
    c->nearinv_ok = 0;
    c->learned = 0;
    c->nearinv_own = own_only;
    long long total = c->nnz;
    if (own_only) {
        std::vector<long long> boff(leaf.nb + 1, 0);
        for (int b = 0; b < leaf.nb; ++b) {
            const long long n = c->box_ptr[b + 1] - c->box_ptr[b];
            boff[b + 1] = boff[b] + n * n;
        }
        total = boff[leaf.nb];
        CK(cudaMalloc(&c->dboff, boff.size() * sizeof(long long)));
        CK(cudaMemcpy(c->dboff, boff.data(), boff.size() * sizeof(long long), cudaMemcpyHostToDevice));
    }
    c->minv_len = total;
    CK(cudaMalloc(&c->dMinv, std::max<long long>(total, 1) * sizeof(double2)));
    // large neighbourhoods: the blocked FP32 LU (mlf_nbhd_lu.cu)
    if (!own_only && (c->nearinv_bits == 32 || (c->nearinv_bits == 0 && nmax > NBI_FP64_MAX))) {
        const int st = nbhd_inverse_lu32(c, nownmax, bad_box);
        if (st) return st;
        c->nearinv_ok = *bad_box == 0;
        return MLF_OK;
    }
    double2* work = nullptr;
    int* dbad = nullptr;
    int* dbases = nullptr;
    CK(ds.alloc(&work, slab * batch * sizeof(double2)));
    CK(ds.alloc(&dbad, sizeof(int)));
    const int big = 0x7fffffff;
    CK(cudaMemcpy(dbad, &big, sizeof(int), cudaMemcpyHostToDevice));
    dbases = c->dperm;   // the box-sorted basis list
    // each box's own bases in ascending order: the box-sorted list already is
    for (int b0 = 0; b0 < leaf.nb; b0 += batch) {
        k_nbhd_inverse<<<std::min(batch, leaf.nb - b0), NBI_THREADS, 0, c->stream>>>(
            b0, leaf.nb, c->dbox_ptr, dbases, dbases, own_only, c->dia, c->dja, c->dZ, slab, work, c->dMinv,
            c->dboff, dbad);
        CK(cudaGetLastError());
    }
    int hbad = 0;
    CK(cudaMemcpyAsync(&hbad, dbad, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    *bad_box = hbad == big ? 0 : hbad;
    c->nearinv_ok = *bad_box == 0;
    return MLF_OK;
}

int device_nearinv_apply(Ctx* c, const double2* y, double2* x, int nrhs, cudaStream_t s) {
    if (!c->nearinv_ok) {
        c->err = "neighbourhood-inverse preconditioner not built (mlf_nearinv has not succeeded)";
        return MLF_E_STATE;
    }
    const long long warps = (long long)c->N * nrhs;
    if (c->nearinv_own)
        k_blockdiag_apply<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, s>>>(
            c->N, nrhs, c->dbox_ptr, c->dbox_of_sorted, c->dperm, c->dboff, c->dMinv, y, x);
    else
        k_spmv_z<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, s>>>(c->N, nrhs, c->dia, c->dja, c->dMinv, y, x);
    return cuda_ok(c, cudaGetLastError(), "nearinv apply") ? MLF_OK : MLF_E_CUDA;
}

}  // namespace mlf

using namespace mlf;

extern "C" int mlf_nearinv(mlf_ctx* h, int* bad_box) {
    if (!h || !bad_box) return MLF_E_ARG;
    Ctx* c = &h->c;
    if (!cuda_ok(c, cudaSetDevice(c->dev), "cudaSetDevice")) return MLF_E_CUDA;
    return device_nearinv_setup(c, bad_box, 0);
}

extern "C" int mlf_nearinv_own(mlf_ctx* h, int* bad_box) {
    if (!h || !bad_box) return MLF_E_ARG;
    Ctx* c = &h->c;
    if (!cuda_ok(c, cudaSetDevice(c->dev), "cudaSetDevice")) return MLF_E_CUDA;
    return device_nearinv_setup(c, bad_box, 1);
}

extern "C" int mlf_set_nearinv_precision(mlf_ctx* h, int bits) {
    if (!h || (bits != 0 && bits != 32 && bits != 64)) return MLF_E_ARG;
    h->c.nearinv_bits = bits;
    return MLF_OK;
}

extern "C" int mlf_nearinv_values(mlf_ctx* h, double* vals) {
    if (!h || !vals) return MLF_E_ARG;
    Ctx* c = &h->c;
    if (!c->nearinv_ok || c->nearinv_own) {
        c->err = "neighbourhood-inverse values exist for the full-neighbourhood mode only";
        return MLF_E_STATE;
    }
    if (!cuda_ok(c, cudaSetDevice(c->dev), "cudaSetDevice")) return MLF_E_CUDA;
    CK(cudaMemcpy(vals, c->dMinv, c->nnz * sizeof(double2), cudaMemcpyDeviceToHost));
    return MLF_OK;
}
