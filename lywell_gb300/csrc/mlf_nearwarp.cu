// Multi-column FP32 operator kernels for meshes with few bases per leaf box
// (block engine 2, the warp engine).
//
// With ten or so bases per leaf box (a sphere meshed at lambda/10 with
// lambda/4 leaves) the 64-row box-block tiles of mlf_nearblk.cu are mostly
// padding.  Here one warp serves one basis for a chunk of NR columns: its
// lanes are NR columns x (32 / NR) near entries, so each near value, pattern
// sample and preconditioner entry is read once per NR columns and nothing is
// padded.  The input block is the box-sorted, row-major copy
// xs[pos * nrhs + r] that device_blk_pack makes; the near CSR's column
// indices are remapped once to sorted positions (jas), so the x rows a warp
// gathers are the contiguous rows of its near boxes, and consecutive warps
// (consecutive bases of one box) gather the same rows.
//
// The sums are those of the single-column kernels (k32_receive_near and
// k32_aggregate: MatxVec_MLFMA / llenar_campoCyB, modMLFMA.f90:1805-1811 and
// 1915-1924; k32_spmv_z and k32_blockdiag_apply for the preconditioners), in
// another order.
#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>

#include "mlf_internal.h"

namespace mlf {

#define CK(call)                                             \
    do {                                                     \
        if (!cuda_ok(c, (call), #call)) return MLF_E_CUDA;   \
    } while (0)

__global__ void k_inverse_perm(int N, const int* __restrict__ perm, int* __restrict__ ipos) {
    const int pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos < N) ipos[perm[pos]] = pos;
}

__global__ void k_sorted_cols(long long nnz, const int* __restrict__ ja, const int* __restrict__ ipos,
                              int* __restrict__ jas) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nnz; q += (long long)gridDim.x * blockDim.x)
        jas[q] = ipos[ja[q]];
}

// Sum over the lanes that share lane % NR (the entry slots of one column).
template <int NR>
__device__ __forceinline__ float slot_sum(float v) {
#pragma unroll
    for (int o = NR; o < 32; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Warp sums of M = 2^m values per lane in M - 1 + (5 - m) shuffles: the first
// m exchanges (offsets 16, 8, ...) each hand half of the remaining values to
// the partner lane and keep the other half, the last 5 - m add plainly.
// Lane L ends with the total of value index (L >> (5 - m)).
template <int M>
__device__ __forceinline__ float warp_split_sum(float (&v)[M], int lane) {
#pragma unroll
    for (int s = 0; s < 5; ++s) {
        const int o = 16 >> s;
        if ((M >> s) > 1) {
            const int h = (M >> s) / 2;
            const bool up = (lane & o) != 0;
#pragma unroll
            for (int i = 0; i < M / 2; ++i) {
                if (i < h) {
                    const float send = up ? v[i] : v[i + h];
                    const float keep = up ? v[i + h] : v[i];
                    v[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
                }
            }
        } else {
            v[0] += __shfl_xor_sync(0xffffffffu, v[0], o);
        }
    }
    return v[0];
}

template <int NR> struct Log2;
template <> struct Log2<1> { static constexpr int v = 0; };
template <> struct Log2<2> { static constexpr int v = 1; };
template <> struct Log2<4> { static constexpr int v = 2; };
template <> struct Log2<8> { static constexpr int v = 3; };

// Near-field sum of CSR row n for column c0 + r over the warp's entry slots
// (lane = slot g x column r), returned summed over the slots in every lane.
// Four entries per lane in flight: each is a chain of two dependent loads
// (the column's sorted position, then x), so unrolling is what hides their
// latency.
template <int NR>
__device__ __forceinline__ void near_row(int n, int g, int r, bool live, int c0, int nrhs,
                                         const int* __restrict__ ia, const int* __restrict__ jas,
                                         const float2* __restrict__ Z, const float2* __restrict__ xs, float& tr,
                                         float& ti) {
    constexpr int G = 32 / NR;
    const float2* xc = xs + c0 + r;
    const int q1 = ia[n + 1];
    int q = ia[n] + g;
    tr = 0.f;
    ti = 0.f;
    for (; q + 3 * G < q1; q += 4 * G) {
        float2 z[4], v[4];
        int j[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) { z[u] = Z[q + u * G]; j[u] = jas[q + u * G]; }
#pragma unroll
        for (int u = 0; u < 4; ++u) v[u] = live ? xc[(size_t)j[u] * nrhs] : make_float2(0.f, 0.f);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            tr = fmaf(z[u].x, v[u].x, tr); tr = fmaf(-z[u].y, v[u].y, tr);
            ti = fmaf(z[u].x, v[u].y, ti); ti = fmaf(z[u].y, v[u].x, ti);
        }
    }
    for (; q < q1; q += G) {
        const float2 z = Z[q];
        const float2 v = live ? xc[(size_t)jas[q] * nrhs] : make_float2(0.f, 0.f);
        tr = fmaf(z.x, v.x, tr); tr = fmaf(-z.y, v.y, tr);
        ti = fmaf(z.x, v.y, ti); ti = fmaf(z.y, v.x, ti);
    }
    tr = slot_sum<NR>(tr);
    ti = slot_sum<NR>(ti);
}

// Receive sum sum_k conj(R_n[k]) A(k, col) for columns c0 .. c0 + NR - 1,
// A(:, u) at Ab + u * K2; lane r ends with column r's (Re, Im).
template <int NR>
__device__ __forceinline__ void recv_row(const float2* __restrict__ Rn, const float2* Ab, int K2, int lane, int r,
                                         int ncol, float& sr, float& si) {
    float v[2 * NR];   // Re, then Im, of sum conj(R) A for each column
#pragma unroll
    for (int u = 0; u < 2 * NR; ++u) v[u] = 0.f;
    for (int k = lane; k < K2; k += 32) {
        const float2 a = Rn[k];
#pragma unroll
        for (int u = 0; u < NR; ++u) {
            if (u < ncol) {
                const float2 w = Ab[(size_t)u * K2 + k];
                v[u] = fmaf(a.x, w.x, v[u]); v[u] = fmaf(a.y, w.y, v[u]);
                v[NR + u] = fmaf(a.x, w.y, v[NR + u]); v[NR + u] = fmaf(-a.y, w.x, v[NR + u]);
            }
        }
    }
    const float s = warp_split_sum<2 * NR>(v, lane);
    constexpr int sh = 5 - (Log2<NR>::v + 1);
    sr = __shfl_sync(0xffffffffu, s, r << sh);
    si = __shfl_sync(0xffffffffu, s, (NR + r) << sh);
}

// For the bases in box-sorted order (one warp each) and columns
// [c0, c0 + NR), c0 = blockIdx.y * NR:
//   t(n, col) = sum_q Z[q] x(ja[q], col)                       (near CSR row n)
//             + j facy sum_k conj(R_n[k]) A_box(n)(k, col)     (when R != null)
// OUT 0: y(n, col) = t in FP64 columns (leading dimension ld), written.
// OUT 1: out32(n, col) = t in FP32 columns (ld), written: a preconditioner
// with the near pattern (R null).
template <int NR, int OUT>
__global__ void __launch_bounds__(256) k32_near_warp(int N, int nrhs, int ld, int K2, float facy,
                                                     const int* __restrict__ perm,
                                                     const int* __restrict__ box_of_sorted,
                                                     const float2* __restrict__ R, const float2* __restrict__ A,
                                                     const int* __restrict__ ia, const int* __restrict__ jas,
                                                     const float2* __restrict__ Z, const float2* __restrict__ xs,
                                                     double2* __restrict__ y, float2* __restrict__ out32) {
    const int pos = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
    if (pos >= N) return;   // whole warps leave together
    const int lane = threadIdx.x & 31;
    const int c0 = blockIdx.y * NR;
    const int g = lane / NR, r = lane % NR;   // entry slot, column
    const bool live = c0 + r < nrhs;
    const int n = perm[pos];
    float tr, ti;
    near_row<NR>(n, g, r, live, c0, nrhs, ia, jas, Z, xs, tr, ti);
    if (OUT == 0 && R) {
        const int b = box_of_sorted[pos];
        float sr, si;
        recv_row<NR>(R + (size_t)pos * K2, A + ((size_t)b * nrhs + c0) * K2, K2, lane, r, nrhs - c0, sr, si);
        tr = fmaf(-facy, si, tr);
        ti = fmaf(facy, sr, ti);
    }
    if (g == 0 && live) {
        if (OUT == 0) y[(size_t)(c0 + r) * ld + n] = make_double2((double)tr, (double)ti);
        else out32[(size_t)(c0 + r) * ld + n] = make_float2(tr, ti);
    }
}

// The same near field + receive with one CTA per leaf box: the box's A
// fields for the NR columns are staged once in shared memory, and the CTA's
// warps walk the box's bases.  The sums are the per-basis kernel's, in the
// same order.
template <int NR>
__global__ void __launch_bounds__(128) k32_nearrecv_box(int nrhs, int ld, int K2, float facy,
                                                        const int* __restrict__ box_ptr,
                                                        const int* __restrict__ perm, const float2* __restrict__ R,
                                                        const float2* __restrict__ A, const int* __restrict__ ia,
                                                        const int* __restrict__ jas, const float2* __restrict__ Z,
                                                        const float2* __restrict__ xs, double2* __restrict__ y) {
    extern __shared__ __align__(16) unsigned char box_smem[];
    float2* As = reinterpret_cast<float2*>(box_smem);   // NR x K2
    const int b = blockIdx.x, c0 = blockIdx.y * NR;
    const float2* Ab = A + ((size_t)b * nrhs + c0) * K2;
    for (int i = threadIdx.x; i < NR * K2; i += blockDim.x) {
        const int u = i / K2;
        As[i] = c0 + u < nrhs ? Ab[i] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int g = lane / NR, r = lane % NR;
    const bool live = c0 + r < nrhs;
    const int j1 = box_ptr[b + 1];
    for (int pos = box_ptr[b] + (threadIdx.x >> 5); pos < j1; pos += nw) {   // warp-uniform
        const int n = perm[pos];
        float tr, ti, sr, si;
        near_row<NR>(n, g, r, live, c0, nrhs, ia, jas, Z, xs, tr, ti);
        recv_row<NR>(R + (size_t)pos * K2, As, K2, lane, r, nrhs - c0, sr, si);
        tr = fmaf(-facy, si, tr);
        ti = fmaf(facy, sr, ti);
        if (g == 0 && live) y[(size_t)(c0 + r) * ld + n] = make_double2((double)tr, (double)ti);
    }
}

// Leaf aggregation for columns [c0, c0 + NR): C(k, col, box) = sum over the
// box's bases t of R_t[k] x(t, col); one CTA per leaf box, threads over the
// 2K samples, each pattern sample read once per NR columns.
template <int NR>
__global__ void __launch_bounds__(128) k32_agg_warp(int K2, int nrhs, const int* __restrict__ box_ptr,
                                                    const float2* __restrict__ R, const float2* __restrict__ xs,
                                                    float2* __restrict__ C) {
    const int b = blockIdx.x, c0 = blockIdx.y * NR;
    const int j0 = box_ptr[b], j1 = box_ptr[b + 1];
    for (int k = threadIdx.x; k < K2; k += blockDim.x) {
        float ax[NR], ay[NR];
#pragma unroll
        for (int u = 0; u < NR; ++u) ax[u] = ay[u] = 0.f;
        int t = j0;
        for (; t + 1 < j1; t += 2) {   // two pattern rows in flight
            const float2 a0 = R[(size_t)t * K2 + k], a1 = R[(size_t)(t + 1) * K2 + k];
            const float2* xv = xs + (size_t)t * nrhs + c0;
#pragma unroll
            for (int u = 0; u < NR; ++u) {
                if (c0 + u < nrhs) {
                    const float2 w = xv[u], w1 = xv[nrhs + u];
                    ax[u] = fmaf(a0.x, w.x, ax[u]); ax[u] = fmaf(-a0.y, w.y, ax[u]);
                    ay[u] = fmaf(a0.x, w.y, ay[u]); ay[u] = fmaf(a0.y, w.x, ay[u]);
                    ax[u] = fmaf(a1.x, w1.x, ax[u]); ax[u] = fmaf(-a1.y, w1.y, ax[u]);
                    ay[u] = fmaf(a1.x, w1.y, ay[u]); ay[u] = fmaf(a1.y, w1.x, ay[u]);
                }
            }
        }
        for (; t < j1; ++t) {
            const float2 a = R[(size_t)t * K2 + k];
            const float2* xv = xs + (size_t)t * nrhs + c0;
#pragma unroll
            for (int u = 0; u < NR; ++u) {
                if (c0 + u < nrhs) {
                    const float2 w = xv[u];
                    ax[u] = fmaf(a.x, w.x, ax[u]); ax[u] = fmaf(-a.y, w.y, ax[u]);
                    ay[u] = fmaf(a.x, w.y, ay[u]); ay[u] = fmaf(a.y, w.x, ay[u]);
                }
            }
        }
#pragma unroll
        for (int u = 0; u < NR; ++u)
            if (c0 + u < nrhs) C[((size_t)b * nrhs + c0 + u) * K2 + k] = make_float2(ax[u], ay[u]);
    }
}

// Own-box block preconditioner for columns [c0, c0 + NR):
// out(n, col) = sum_t M_box[i][t] x(box basis t, col), M row-major n_b x n_b
// at boff[box], i the basis's place in its box; one warp per basis.
template <int NR>
__global__ void __launch_bounds__(256) k32_own_warp(int N, int nrhs, const int* __restrict__ box_ptr,
                                                    const int* __restrict__ box_of_sorted,
                                                    const int* __restrict__ perm, const long long* __restrict__ boff,
                                                    const float2* __restrict__ M, const float2* __restrict__ xs,
                                                    float2* __restrict__ out) {
    const int pos = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
    if (pos >= N) return;
    const int lane = threadIdx.x & 31;
    const int c0 = blockIdx.y * NR;
    const int g = lane / NR, r = lane % NR;
    const bool live = c0 + r < nrhs;
    const int b = box_of_sorted[pos], j0 = box_ptr[b], nb = box_ptr[b + 1] - j0;
    const float2* row = M + boff[b] + (size_t)(pos - j0) * nb;
    const float2* xc = xs + (size_t)j0 * nrhs + c0 + r;
    float tr = 0.f, ti = 0.f;
    for (int t = g; t < nb; t += 32 / NR) {
        const float2 a = row[t];
        const float2 v = live ? xc[(size_t)t * nrhs] : make_float2(0.f, 0.f);
        tr = fmaf(a.x, v.x, tr); tr = fmaf(-a.y, v.y, tr);
        ti = fmaf(a.x, v.y, ti); ti = fmaf(a.y, v.x, ti);
    }
    tr = slot_sum<NR>(tr);
    ti = slot_sum<NR>(ti);
    if (g == 0 && live) out[(size_t)(c0 + r) * N + perm[pos]] = make_float2(tr, ti);
}

// jas: the near CSR's column indices as box-sorted positions (built once)
static int warp_setup(Ctx* c) {
    if (c->djas) return MLF_OK;
    if (need_tree(c)) return MLF_E_STATE;
    DevScope ds;
    int* ipos = nullptr;
    CK(ds.alloc(&ipos, std::max(c->N, 1) * sizeof(int)));
    CK(cudaMalloc(&c->djas, std::max<long long>(c->nnz, 1) * sizeof(int)));
    k_inverse_perm<<<(c->N + 255) / 256, 256, 0, c->stream>>>(c->N, c->dperm, ipos);
    if (c->nnz)
        k_sorted_cols<<<(unsigned)std::min<long long>((c->nnz + 255) / 256, 65535), 256, 0, c->stream>>>(
            c->nnz, c->dja, ipos, c->djas);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->stream));   // before ipos is freed
    return MLF_OK;
}

// The engine in force: the one set (mlf_set_block_engine, the autotuner),
// else the warp engine when leaf boxes hold fewer than 48 bases on average.
int blk_engine_of(const Ctx* c) {
    if (c->blk_engine >= 0) return c->blk_engine;
    const long long nb = (long long)c->box_ptr.size() - 1;
    return (nb > 0 && c->N < 48LL * nb) ? 2 : 1;
}

// columns per warp pass: the block's width rounded up to 1, 2, 4 or 8
static int warp_nr(int nrhs) { return nrhs <= 1 ? 1 : nrhs <= 2 ? 2 : nrhs <= 4 ? 4 : 8; }

template <class F>
static void nr_dispatch(int nrhs, F f) {
    switch (warp_nr(nrhs)) {
        case 1: f(std::integral_constant<int, 1>()); break;
        case 2: f(std::integral_constant<int, 2>()); break;
        case 4: f(std::integral_constant<int, 4>()); break;
        default: f(std::integral_constant<int, 8>()); break;
    }
}

// C (leaf fields) = R^T x
int device_agg_warp32(Ctx* c, const float2* R, int K, const float2* xs, int nrhs, float2* C, cudaStream_t s) {
    const int nb = (int)c->box_ptr.size() - 1;
    nr_dispatch(nrhs, [&](auto nr) {
        constexpr int NR = decltype(nr)::value;
        k32_agg_warp<NR><<<dim3(nb, (nrhs + NR - 1) / NR), 128, 0, s>>>(2 * K, nrhs, c->dbox_ptr, R, xs, C);
    });
    return cuda_ok(c, cudaGetLastError(), "aggregation (warp)") ? MLF_OK : MLF_E_CUDA;
}

// y = Z_near x + j facy conj(R) A (leaf receive), written
int device_recv_near_warp32(Ctx* c, const float2* R, int K, const float2* A, float facy, const float2* xs, int nrhs,
                            int ld, double2* y, cudaStream_t s) {
    int st;
    if ((st = warp_setup(c))) return st;
    const unsigned grid = (unsigned)(((size_t)c->N * 32 + 255) / 256);
    const int nb = (int)c->box_ptr.size() - 1;
    nr_dispatch(nrhs, [&](auto nr) {
        constexpr int NR = decltype(nr)::value;
        const size_t smem = (size_t)NR * 2 * K * sizeof(float2);
        if (blk_engine_of(c) == 2 && smem <= 48 * 1024)   // the box's A fields in shared memory
            k32_nearrecv_box<NR><<<dim3(nb, (nrhs + NR - 1) / NR), 128, smem, s>>>(
                nrhs, ld, 2 * K, facy, c->dbox_ptr, c->dperm, R, A, c->dia, c->djas, c->dZ, xs, y);
        else
            k32_near_warp<NR, 0><<<dim3(grid, (nrhs + NR - 1) / NR), 256, 0, s>>>(
                c->N, nrhs, ld, 2 * K, facy, c->dperm, c->dbox_of_sorted, R, A, c->dia, c->djas, c->dZ, xs, y,
                nullptr);
    });
    return cuda_ok(c, cudaGetLastError(), "near + receive (warp)") ? MLF_OK : MLF_E_CUDA;
}

// out (FP32 columns, ld N) = M xs for M in CSR form with the near pattern
int device_near_pattern_warp32(Ctx* c, const float2* M, const float2* xs, int nrhs, float2* out, cudaStream_t s) {
    int st;
    if ((st = warp_setup(c))) return st;
    const unsigned grid = (unsigned)(((size_t)c->N * 32 + 255) / 256);
    nr_dispatch(nrhs, [&](auto nr) {
        constexpr int NR = decltype(nr)::value;
        k32_near_warp<NR, 1><<<dim3(grid, (nrhs + NR - 1) / NR), 256, 0, s>>>(
            c->N, nrhs, c->N, 0, 0.f, c->dperm, c->dbox_of_sorted, nullptr, nullptr, c->dia, c->djas, M, xs, nullptr,
            out);
    });
    return cuda_ok(c, cudaGetLastError(), "near-pattern apply (warp)") ? MLF_OK : MLF_E_CUDA;
}

// out (FP32 columns, ld N) = own-box blocks M applied to xs
int device_own_warp32(Ctx* c, const long long* boff, const float2* M, const float2* xs, int nrhs, float2* out,
                      cudaStream_t s) {
    if (need_tree(c)) return MLF_E_STATE;
    const unsigned grid = (unsigned)(((size_t)c->N * 32 + 255) / 256);
    nr_dispatch(nrhs, [&](auto nr) {
        constexpr int NR = decltype(nr)::value;
        k32_own_warp<NR><<<dim3(grid, (nrhs + NR - 1) / NR), 256, 0, s>>>(c->N, nrhs, c->dbox_ptr,
                                                                          c->dbox_of_sorted, c->dperm, boff, M, xs,
                                                                          out);
    });
    return cuda_ok(c, cudaGetLastError(), "own-box apply (warp)") ? MLF_OK : MLF_E_CUDA;
}

void warp_engine_free(Ctx* c) {
    if (c->djas) cudaFree(c->djas);
    c->djas = nullptr;
}

}  // namespace mlf
