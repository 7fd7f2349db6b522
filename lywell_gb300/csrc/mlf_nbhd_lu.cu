// Neighbourhood-inverse preconditioner for large neighbourhoods: a blocked,
// FP32, partially pivoted LU per leaf box.
//
// The preconditioner (mlf_precond.cu) needs, for every leaf box b, the rows of
// inv(A) that belong to b's own bases, A = Znear[S, S] over the box's near
// list S.  Its FP64 elimination works by rank-1 updates of A in global memory,
// which is fine for neighbourhoods of a few hundred unknowns but not for the
// 1500-4000 unknowns of bodies with 60-150 bases per 0.25 lambda leaf box
// (the prolate spheroid of the 722-RHS workload, the superellipsoids of the
// learned preconditioner): there the work is ~2.7 n^3 flops per box and the
// rank-1 form re-reads the whole matrix n times.
//
// This kernel solves the same system, A^T X = E_own (then M rows = X^T), with
// a right-looking blocked LU of A^T, column-major in a per-CTA slab of global
// memory (L2-resident in part):
//   for each panel of LU_P = 32 columns:
//     * panel factorisation: pivot = largest |a|^2 at or below the diagonal
//       (first row on ties), row swap across the trailing columns and X,
//       scaling, rank-1 updates inside the panel;
//     * U12 = L11^-1 A12 for the trailing columns and the right-hand sides X
//       (forward substitution on 32 x 64 tiles in shared memory, one thread
//       per column);
//     * trailing update A22 -= L21 U12 and X2 -= L21 X1 by strips of 64
//       rows: a register-blocked FP32 GEMM over 64 x 64 complex tiles (each
//       thread 2 x 8 outputs), L staged once per strip, the next U tile and
//       the current output tile loaded while the FMAs run;
//   back substitution U X = Y by blocks of 32 rows from the bottom (a small
//   triangular solve per block, then a tiled GEMM update of the rows above).
// Persistent CTAs (two per SM) take boxes from an atomic counter, largest
// neighbourhoods first, so large and small neighbourhoods balance over the GPU.
//
// The same kernel computes the learned preconditioner's training targets
// (mlf_learned.cu): rows of the inverse over each box's 2-ring (125-box)
// neighbourhood, the system taken from a dense Z.
//
// FP32 with partial pivoting leaves the preconditioner's rows within ~1e-5 of
// the FP64 ones (tested); a preconditioner only has to be close, and the
// solves' residual test stays FP64.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "mlf_internal.h"

namespace mlf {

#define CK(call)                                             \
    do {                                                     \
        if (!cuda_ok(c, (call), #call)) return MLF_E_CUDA;   \
    } while (0)

constexpr int LU_P = 32;          // panel width (= block of the back substitution)
constexpr int LU_T = 64;          // GEMM tile rows and columns
constexpr int LU_THREADS = 256;
constexpr int LU_BIG_MAX = 512;       // boxes at most on the many-CTA path
constexpr int LU_BIG_STREAMS = 8;     // large boxes in flight at once
constexpr double LU_BIG_FACTOR = 3.0; // a box goes to the many-CTA path above this many CTA shares

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cinvf(float2 a) {
    const float d = a.x * a.x + a.y * a.y;
    return make_float2(a.x / d, -a.y / d);
}

__device__ __forceinline__ int bsearch_cols(const int* S, int n, int v) {
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

// One 64-row strip of D -= Lop * Uop over K = kb, 64 columns at a time:
//   Lop(i, t) = A[(lk + t) * n + lr + r0 + i]                     (column-major panel)
//   Uop(t, j) = col(j)[uk + t],  col(q) = q < nc ? A + (ac + q) * n : X + (q - nc) * n
//   D(i, j)   = col(j)[dr + r0 + i]
// rows r0 .. r0+63 (< nrows), columns cbeg .. cend-1.  The L tile is staged
// once per strip; while a column tile is multiplied, the next tile's U values
// and the current tile's D values are already in flight (registers), so the
// loads overlap the FMAs.  Warp w owns columns 8w .. 8w+7 of a tile and each
// lane rows lane and lane + 32: the U values are warp-wide broadcasts and the
// D accesses coalesced.  The caller synchronises before; this ends synchronised.
// The 2-ring variant (training targets of the learned preconditioner): the
// system comes from a dense Z (complex(4), row-major N x N) over each box's
// sorted 2-ring list, and the rows go to M2 on the near pattern.  Zd null:
// the near-list variant.
struct LuRing {
    const float2* Zd = nullptr;
    int N = 0;
    const long long* off = nullptr;
    const int* len = nullptr;
    const int* bases = nullptr;
    float2* M2 = nullptr;
};

struct LuTiles {
    float2 L[LU_T][LU_P + 1];
    float2 U[2][LU_P][LU_T + 1];
};

struct LuShared {
    LuTiles t;
    float val[LU_THREADS / 32];
    int idx[LU_THREADS / 32];
    int piv, sing;
    float2 u[LU_P];
};

__device__ __forceinline__ float2* lu_col(float2* A, float2* X, int n, int ac, int nc, int q) {
    return q < nc ? A + (size_t)(ac + q) * n : X + (size_t)(q - nc) * n;
}

__device__ __forceinline__ void lu_strip_update(LuTiles& sm, float2* __restrict__ A, float2* __restrict__ X, int n,
                                                int kb, int lk, int lr, int uk, int dr, int ac, int nc, int r0,
                                                int nrows, int cbeg, int cend) {
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    constexpr int PER = LU_T * LU_P / LU_THREADS;   // U values per thread per tile (8)
#pragma unroll
    for (int e = tid; e < LU_T * LU_P; e += LU_THREADS) {
        const int t = e / LU_T, i = e - t * LU_T;          // consecutive threads: consecutive rows
        sm.L[i][t] = (t < kb && r0 + i < nrows) ? A[(size_t)(lk + t) * n + lr + r0 + i] : make_float2(0.f, 0.f);
    }
    float2 un[PER];
    auto load_u = [&](int c0) {
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            const int e = tid + k * LU_THREADS;
            const int j = e / LU_P, t = e - j * LU_P;      // consecutive threads: consecutive t of one column
            un[k] = (t < kb && c0 + j < cend) ? lu_col(A, X, n, ac, nc, c0 + j)[uk + t] : make_float2(0.f, 0.f);
        }
    };
    auto stage_u = [&](int buf) {
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            const int e = tid + k * LU_THREADS;
            const int j = e / LU_P, t = e - j * LU_P;
            sm.U[buf][t][j] = un[k];
        }
    };
    load_u(cbeg);
    stage_u(0);
    __syncthreads();
    int buf = 0;
    for (int c0 = cbeg; c0 < cend; c0 += LU_T) {
        // in flight during the FMAs: the next tile's U values and this tile's D values
        if (c0 + LU_T < cend) load_u(c0 + LU_T);
        float2 d[2][8];
#pragma unroll
        for (int v = 0; v < 8; ++v) {
            const int q = c0 + 8 * w + v;
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int i = lane + 32 * u;
                d[u][v] = (q < cend && r0 + i < nrows) ? lu_col(A, X, n, ac, nc, q)[dr + r0 + i]
                                                       : make_float2(0.f, 0.f);
            }
        }
        // the K-sum accumulates on its own and is subtracted once (the
        // in-place form rounds each product against the larger D value)
        float2 acc[2][8];
#pragma unroll
        for (int u = 0; u < 2; ++u)
#pragma unroll
            for (int v = 0; v < 8; ++v) acc[u][v] = make_float2(0.f, 0.f);
        for (int t = 0; t < kb; ++t) {
            const float2 a0 = sm.L[lane][t], a1 = sm.L[lane + 32][t];
#pragma unroll
            for (int v = 0; v < 8; ++v) {
                const float2 b = sm.U[buf][t][8 * w + v];
                acc[0][v].x = fmaf(a0.x, b.x, acc[0][v].x);
                acc[0][v].x = fmaf(-a0.y, b.y, acc[0][v].x);
                acc[0][v].y = fmaf(a0.x, b.y, acc[0][v].y);
                acc[0][v].y = fmaf(a0.y, b.x, acc[0][v].y);
                acc[1][v].x = fmaf(a1.x, b.x, acc[1][v].x);
                acc[1][v].x = fmaf(-a1.y, b.y, acc[1][v].x);
                acc[1][v].y = fmaf(a1.x, b.y, acc[1][v].y);
                acc[1][v].y = fmaf(a1.y, b.x, acc[1][v].y);
            }
        }
#pragma unroll
        for (int v = 0; v < 8; ++v) {
            const int q = c0 + 8 * w + v;
            if (q >= cend) continue;
            float2* col = lu_col(A, X, n, ac, nc, q);
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int i = lane + 32 * u;
                if (r0 + i < nrows) col[dr + r0 + i] = make_float2(d[u][v].x - acc[u][v].x, d[u][v].y - acc[u][v].y);
            }
        }
        if (c0 + LU_T < cend) stage_u(buf ^ 1);
        __syncthreads();
        buf ^= 1;
    }
}

// ---- the phases of one box's solve, each executed by the CTAs part = 0 ..
// nparts-1 over disjoint pieces (one CTA: part 0 of 1, all of it)

// A^T column r = row S[r] of Z restricted to S; X = the own bases' unit columns.
// zeroed: A and X are already zero (else part 0 of 1 zeroes them first).
__device__ void lu_assemble(float2* A, float2* X, int b, int n, int nown, const int* S, const int* box_ptr,
                            const int* box_bases, const int* ia, const int* ja, const float2* Z, const LuRing& ring,
                            bool zeroed, int part, int nparts) {
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const size_t g0 = (size_t)part * LU_THREADS + tid, gs = (size_t)nparts * LU_THREADS;
    if (ring.Zd) {
        for (size_t e = g0; e < (size_t)n * n; e += gs) {
            const int r = (int)(e / n), pos = (int)(e - (size_t)r * n);
            A[e] = ring.Zd[(size_t)S[r] * ring.N + S[pos]];
        }
        if (!zeroed) {
            for (size_t e = g0; e < (size_t)n * nown; e += gs) X[e] = make_float2(0.f, 0.f);
            __syncthreads();
        }
    } else {
        if (!zeroed) {
            for (size_t e = g0; e < (size_t)n * n + (size_t)n * nown; e += gs) A[e] = make_float2(0.f, 0.f);
            __syncthreads();
        }
        for (int r = part * (LU_THREADS / 32) + wid; r < n; r += nparts * (LU_THREADS / 32)) {
            const int m = S[r];
            for (int q = ia[m] + lane; q < ia[m + 1]; q += 32) {
                const int pos = bsearch_cols(S, n, ja[q]);
                if (pos >= 0) A[(size_t)r * n + pos] = Z[q];
            }
        }
    }
    for (int cc = (int)g0; cc < nown; cc += (int)gs) {
        const int pos = bsearch_cols(S, n, box_bases[box_ptr[b] + cc]);
        if (pos >= 0) X[(size_t)cc * n + pos] = make_float2(1.f, 0.f);
    }
}

// Panel factorisation of columns k0 .. k0+kb-1 (one CTA): pivot = largest
// |a|^2 at or below the diagonal (first row on ties), the row swap applied to
// the columns k0 .. swap_end-1 of the set [A, X] (the trailing columns and X
// now, or only the panel when piv records the pivots for a later swap),
// scaling, rank-1 updates inside the panel.  Returns false when singular.
__device__ bool lu_panel(LuShared& sh, float2* A, float2* X, int n, int k0, int kb, int swap_end, int* piv) {
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    for (int j = k0; j < k0 + kb; ++j) {
        float best = -1.f;
        int bi = n;
        const float2* colj = A + (size_t)j * n;
        for (int i0 = j + tid; i0 < n; i0 += 4 * LU_THREADS) {   // four loads in flight per thread
            float2 a[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int i = i0 + u * LU_THREADS;
                a[u] = i < n ? colj[i] : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int i = i0 + u * LU_THREADS;
                const float v = a[u].x * a[u].x + a[u].y * a[u].y;
                if (i < n && v > best) { best = v; bi = i; }
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const float ov = __shfl_xor_sync(0xffffffffu, best, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
        }
        if (lane == 0) { sh.val[wid] = best; sh.idx[wid] = bi; }
        __syncthreads();
        if (tid == 0) {
            float bv = sh.val[0];
            int bx = sh.idx[0];
            for (int w = 1; w < LU_THREADS / 32; ++w)
                if (sh.val[w] > bv || (sh.val[w] == bv && sh.idx[w] < bx)) { bv = sh.val[w]; bx = sh.idx[w]; }
            sh.piv = bx;
            sh.sing = !(bv > 0.f) || bx >= n;
            if (piv) piv[j - k0] = bx;
        }
        __syncthreads();
        if (sh.sing) return false;
        const int pv = sh.piv;
        if (pv != j) {
            for (int cc = k0 + tid; cc < swap_end; cc += LU_THREADS) {
                float2* col = cc < n ? A + (size_t)cc * n : X + (size_t)(cc - n) * n;
                const float2 t = col[j];
                col[j] = col[pv];
                col[pv] = t;
            }
            __syncthreads();
        }
        const float2 dinv = cinvf(A[(size_t)j * n + j]);
        for (int i = j + 1 + tid; i < n; i += LU_THREADS) {
            float2* p = A + (size_t)j * n + i;
            *p = cmulf(*p, dinv);
        }
        __syncthreads();
        // rank-1 update of the panel's remaining columns: each thread takes rows,
        // the row-j values of those columns staged in shared memory, eight
        // columns' loads in flight at a time
        const int ncl = k0 + kb - j - 1;
        if (tid < ncl) sh.u[tid] = A[(size_t)(j + 1 + tid) * n + j];
        __syncthreads();
        for (int i = j + 1 + tid; i < n; i += LU_THREADS) {
            const float2 l = A[(size_t)j * n + i];
            for (int cq0 = 0; cq0 < ncl; cq0 += 8) {
                float2 d[8];
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    if (cq0 + u < ncl) d[u] = A[(size_t)(j + 1 + cq0 + u) * n + i];
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    if (cq0 + u < ncl) {
                        const float2 uu = sh.u[cq0 + u];
                        d[u].x -= l.x * uu.x - l.y * uu.y;
                        d[u].y -= l.x * uu.y + l.y * uu.x;
                        A[(size_t)(j + 1 + cq0 + u) * n + i] = d[u];
                    }
            }
        }
        __syncthreads();
    }
    return true;
}

// the panel's row swaps on the columns k0+kb .. n+nown-1 of [A, X], in pivot order
__device__ void lu_swap_rest(float2* A, float2* X, int n, int nown, int k0, int kb, const int* piv, int part,
                             int nparts) {
    for (int cc = k0 + kb + part * LU_THREADS + threadIdx.x; cc < n + nown; cc += nparts * LU_THREADS) {
        float2* col = cc < n ? A + (size_t)cc * n : X + (size_t)(cc - n) * n;
        for (int j = k0; j < k0 + kb; ++j) {
            const int p = piv[j - k0];
            if (p != j) {
                const float2 t = col[j];
                col[j] = col[p];
                col[p] = t;
            }
        }
    }
}

// U12 = L11^-1 A12 (and X), unit lower L11 in shared memory, over the column
// tiles part, part + nparts, ... of the trailing columns and X
__device__ void lu_u12(LuTiles& sm, float2* A, float2* X, int n, int nown, int k0, int kb, int part, int nparts) {
    const int tid = threadIdx.x;
    const int nc = n - k0 - kb, ncols = nc + nown;
    for (int e = tid; e < LU_P * LU_P; e += LU_THREADS) {
        const int t = e / LU_P, r = e - t * LU_P;
        sm.L[r][t] = (r < kb && t < kb) ? A[(size_t)(k0 + t) * n + k0 + r] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    for (int c0 = part * LU_T; c0 < ncols; c0 += nparts * LU_T) {
        // a 32 x 64 tile of the columns in shared memory, forward substitution per column
        for (int e = tid; e < LU_T * LU_P; e += LU_THREADS) {
            const int j = e / LU_P, t = e - j * LU_P;
            float2 v = make_float2(0.f, 0.f);
            if (t < kb && c0 + j < ncols) {
                const int q = c0 + j;
                v = (q < nc ? A + (size_t)(k0 + kb + q) * n : X + (size_t)(q - nc) * n)[k0 + t];
            }
            sm.U[0][t][j] = v;
        }
        __syncthreads();
        if (tid < LU_T) {
            for (int r = 1; r < kb; ++r) {
                float2 acc = sm.U[0][r][tid];
                for (int t = 0; t < r; ++t) {
                    const float2 l = sm.L[r][t], u = sm.U[0][t][tid];
                    acc.x -= l.x * u.x - l.y * u.y;
                    acc.y -= l.x * u.y + l.y * u.x;
                }
                sm.U[0][r][tid] = acc;
            }
        }
        __syncthreads();
        for (int e = tid; e < LU_T * LU_P; e += LU_THREADS) {
            const int j = e / LU_P, t = e - j * LU_P;
            if (t < kb && c0 + j < ncols) {
                const int q = c0 + j;
                (q < nc ? A + (size_t)(k0 + kb + q) * n : X + (size_t)(q - nc) * n)[k0 + t] = sm.U[0][t][j];
            }
        }
        __syncthreads();
    }
}

// back substitution of block k0 (rows k0 .. k0+kb-1 of X, U11 from A) over the
// X column tiles part, part + nparts, ...
__device__ void lu_back_block(LuTiles& sm, const float2* A, float2* X, int n, int nown, int k0, int kb, int part,
                              int nparts) {
    const int tid = threadIdx.x;
    for (int e = tid; e < LU_P * LU_P; e += LU_THREADS) {
        const int t = e / LU_P, r = e - t * LU_P;
        sm.L[r][t] = (r < kb && t < kb) ? A[(size_t)(k0 + t) * n + k0 + r] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    for (int c0 = part * LU_T; c0 < nown; c0 += nparts * LU_T) {
        // a 32 x 64 tile of X in shared memory, backward substitution per column
        for (int e = tid; e < LU_T * LU_P; e += LU_THREADS) {
            const int j = e / LU_P, t = e - j * LU_P;
            sm.U[0][t][j] = (t < kb && c0 + j < nown) ? X[(size_t)(c0 + j) * n + k0 + t] : make_float2(0.f, 0.f);
        }
        __syncthreads();
        if (tid < LU_T) {
            for (int r = kb - 1; r >= 0; --r) {
                float2 acc = sm.U[0][r][tid];
                for (int t = r + 1; t < kb; ++t) {
                    const float2 u = sm.L[r][t], x = sm.U[0][t][tid];
                    acc.x -= u.x * x.x - u.y * x.y;
                    acc.y -= u.x * x.y + u.y * x.x;
                }
                sm.U[0][r][tid] = cmulf(acc, cinvf(sm.L[r][r]));
            }
        }
        __syncthreads();
        for (int e = tid; e < LU_T * LU_P; e += LU_THREADS) {
            const int j = e / LU_P, t = e - j * LU_P;
            if (t < kb && c0 + j < nown) X[(size_t)(c0 + j) * n + k0 + t] = sm.U[0][t][j];
        }
        __syncthreads();
    }
}

// rows of the own bases: M[ia[g] + j] = X(j, own index) over the near list,
// or (2-ring) the entries of the near pattern inside the ring list
__device__ void lu_extract(const float2* X, int b, int n, int nown, const int* S, const int* box_ptr,
                           const int* box_bases, const int* ia, const int* ja, double2* M, const LuRing& ring,
                           int part, int nparts) {
    for (int cc = part; cc < nown; cc += nparts) {
        const int g = box_bases[box_ptr[b] + cc];
        const float2* col = X + (size_t)cc * n;
        if (ring.Zd) {
            for (int q = ia[g] + threadIdx.x; q < ia[g + 1]; q += LU_THREADS) {
                const int pos = bsearch_cols(S, n, ja[q]);
                ring.M2[q] = pos >= 0 ? col[pos] : make_float2(0.f, 0.f);
            }
        } else {
            double2* row = M + ia[g];
            for (int j = threadIdx.x; j < n; j += LU_THREADS) row[j] = make_double2((double)col[j].x, (double)col[j].y);
        }
    }
}

__device__ __forceinline__ void lu_box(int b, const int* box_ptr, const int* ia, const LuRing& ring, int box0,
                                       int& n, int& nown, const int*& S, const int* ja) {
    const int m0 = box0;
    nown = box_ptr[b + 1] - box_ptr[b];
    // the neighbourhood: the near list (the CSR row of the box's bases) or the 2-ring list
    n = ring.Zd ? ring.len[b] : ia[m0 + 1] - ia[m0];
    S = ring.Zd ? ring.bases + ring.off[b] : ja + ia[m0];
}

// One CTA per box, persistent: CTAs take boxes from an atomic counter in the
// given order (largest neighbourhoods first).
__global__ void __launch_bounds__(LU_THREADS, 2)
    k_nbhd_lu32(int nb, const int* __restrict__ box_ptr, const int* __restrict__ box_bases,
                const int* __restrict__ ia, const int* __restrict__ ja, const float2* __restrict__ Z, size_t slab,
                float2* __restrict__ work, double2* __restrict__ M, const int* __restrict__ order,
                int* __restrict__ next_box, int* __restrict__ bad, const LuRing ring) {
    __shared__ LuShared sh;
    __shared__ int s_b;
    const int tid = threadIdx.x;
    float2* A = work + (size_t)blockIdx.x * slab;
    for (;;) {
        if (tid == 0) {
            const int k = atomicAdd(next_box, 1);
            s_b = k < nb ? order[k] : -1;      // largest neighbourhoods first
        }
        __syncthreads();
        const int b = s_b;
        if (b < 0) break;
        int n, nown;
        const int* S;
        lu_box(b, box_ptr, ia, ring, box_bases[box_ptr[b]], n, nown, S, ja);
        float2* X = A + (size_t)n * n;
        lu_assemble(A, X, b, n, nown, S, box_ptr, box_bases, ia, ja, Z, ring, false, 0, 1);
        __syncthreads();
        bool ok = true;
        for (int k0 = 0; k0 < n && ok; k0 += LU_P) {
            const int kb = min(LU_P, n - k0);
            ok = lu_panel(sh, A, X, n, k0, kb, n + nown, nullptr);
            if (!ok) break;
            lu_u12(sh.t, A, X, n, nown, k0, kb, 0, 1);
            // trailing update: rows k0+kb.. of the trailing columns and of X
            const int nrows = n - k0 - kb, nc = nrows;
            for (int r0 = 0; r0 < nrows; r0 += LU_T)
                lu_strip_update(sh.t, A, X, n, kb, k0, k0 + kb, k0, k0 + kb, k0 + kb, nc, r0, nrows, 0, nc + nown);
        }
        if (!ok) {
            if (tid == 0) atomicMin(bad, b + 1);
            __syncthreads();
            continue;
        }
        // back substitution U X = Y, blocks of LU_P rows from the bottom
        for (int k0 = ((n - 1) / LU_P) * LU_P; k0 >= 0; k0 -= LU_P) {
            const int kb = min(LU_P, n - k0);
            lu_back_block(sh.t, A, X, n, nown, k0, kb, 0, 1);
            // rows 0..k0-1 of X -= U(0..k0-1, k0..k0+kb-1) X(k0..k0+kb-1)
            for (int r0 = 0; r0 < k0; r0 += LU_T) lu_strip_update(sh.t, A, X, n, kb, k0, 0, k0, 0, 0, 0, r0, k0, 0, nown);
        }
        lu_extract(X, b, n, nown, S, box_ptr, box_bases, ia, ja, M, ring, 0, 1);
        __syncthreads();
    }
}

// ---- one large box on many CTAs: the same phases as kernels, a launch per
// phase and panel on the box's stream (every kernel returns at once once the
// box is singular, *sing set by its panel)

struct LuBig {
    int b, n, nown;
    const int* S;      // device pointer into ja or the 2-ring lists
    float2* A;
    float2* X;
    int* piv;          // LU_P pivots of the current panel
    int* sing;
};

__global__ void __launch_bounds__(LU_THREADS) k_lub_assemble(LuBig g, const int* __restrict__ box_ptr,
                                                             const int* __restrict__ box_bases,
                                                             const int* __restrict__ ia, const int* __restrict__ ja,
                                                             const float2* __restrict__ Z, const LuRing ring) {
    lu_assemble(g.A, g.X, g.b, g.n, g.nown, g.S, box_ptr, box_bases, ia, ja, Z, ring, true, blockIdx.x, gridDim.x);
}

__global__ void __launch_bounds__(LU_THREADS) k_lub_panel(LuBig g, int k0, int* __restrict__ bad) {
    __shared__ LuShared sh;
    if (*reinterpret_cast<volatile int*>(g.sing)) return;
    const int kb = min(LU_P, g.n - k0);
    if (!lu_panel(sh, g.A, g.X, g.n, k0, kb, k0 + kb, g.piv) && threadIdx.x == 0) {
        *g.sing = 1;
        atomicMin(bad, g.b + 1);
    }
}

__global__ void __launch_bounds__(LU_THREADS) k_lub_swap(LuBig g, int k0) {
    if (*reinterpret_cast<volatile int*>(g.sing)) return;
    lu_swap_rest(g.A, g.X, g.n, g.nown, k0, min(LU_P, g.n - k0), g.piv, blockIdx.x, gridDim.x);
}

__global__ void __launch_bounds__(LU_THREADS) k_lub_u12(LuBig g, int k0) {
    __shared__ LuTiles sm;
    if (*reinterpret_cast<volatile int*>(g.sing)) return;
    lu_u12(sm, g.A, g.X, g.n, g.nown, k0, min(LU_P, g.n - k0), blockIdx.x, gridDim.x);
}

// trailing update: CTA (strip blockIdx.x, column chunk blockIdx.y of cw columns)
__global__ void __launch_bounds__(LU_THREADS, 2) k_lub_trail(LuBig g, int k0, int cw) {
    __shared__ LuTiles sm;
    if (*reinterpret_cast<volatile int*>(g.sing)) return;
    const int n = g.n, kb = min(LU_P, n - k0);
    const int nrows = n - k0 - kb, nc = nrows, ncols = nc + g.nown;
    const int r0 = blockIdx.x * LU_T, cb = blockIdx.y * cw;
    if (r0 >= nrows || cb >= ncols) return;
    lu_strip_update(sm, g.A, g.X, n, kb, k0, k0 + kb, k0, k0 + kb, k0 + kb, nc, r0, nrows, cb, min(ncols, cb + cw));
}

__global__ void __launch_bounds__(LU_THREADS) k_lub_back(LuBig g, int k0) {
    __shared__ LuTiles sm;
    if (*reinterpret_cast<volatile int*>(g.sing)) return;
    lu_back_block(sm, g.A, g.X, g.n, g.nown, k0, min(LU_P, g.n - k0), blockIdx.x, gridDim.x);
}

// rows 0..k0-1 of X -= U(0..k0-1, block k0) X(block k0): CTA per (strip, 64 X columns)
__global__ void __launch_bounds__(LU_THREADS, 2) k_lub_back_upd(LuBig g, int k0) {
    __shared__ LuTiles sm;
    if (*reinterpret_cast<volatile int*>(g.sing)) return;
    const int kb = min(LU_P, g.n - k0);
    const int r0 = blockIdx.x * LU_T, cb = blockIdx.y * LU_T;
    if (r0 >= k0 || cb >= g.nown) return;
    lu_strip_update(sm, g.A, g.X, g.n, kb, k0, 0, k0, 0, 0, 0, r0, k0, cb, min(g.nown, cb + LU_T));
}

__global__ void __launch_bounds__(LU_THREADS) k_lub_extract(LuBig g, const int* __restrict__ box_ptr,
                                                            const int* __restrict__ box_bases,
                                                            const int* __restrict__ ia, const int* __restrict__ ja,
                                                            double2* __restrict__ M, const LuRing ring) {
    if (*reinterpret_cast<volatile int*>(g.sing)) return;
    lu_extract(g.X, g.b, g.n, g.nown, g.S, box_ptr, box_bases, ia, ja, M, ring, blockIdx.x, gridDim.x);
}

// One large box on many CTAs, launched on stream s (slab: A and X of the box;
// piv, sing: device scratch of the stream).
static int big_box_launch(Ctx* c, const LuRing& ring, int b, int n, int nown, const int* S, float2* slab, int* piv,
                          int* sing, int* bad, cudaStream_t s) {
    LuBig g{b, n, nown, S, slab, slab + (size_t)n * n, piv, sing};
    CK(cudaMemsetAsync(sing, 0, sizeof(int), s));
    CK(cudaMemsetAsync(slab, 0, ((size_t)n * n + (size_t)n * nown) * sizeof(float2), s));
    const unsigned ga = (unsigned)std::min<long long>(4096, ((long long)n * n + LU_THREADS - 1) / LU_THREADS);
    k_lub_assemble<<<ga, LU_THREADS, 0, s>>>(g, c->dbox_ptr, c->dperm, c->dia, c->dja, c->dZ, ring);
    // trailing-update column chunks: about 8 CTAs' worth of strips per SM in all
    for (int k0 = 0; k0 < n; k0 += LU_P) {
        const int kb = std::min(LU_P, n - k0);
        const int nrows = n - k0 - kb, ncols = nrows + nown;
        k_lub_panel<<<1, LU_THREADS, 0, s>>>(g, k0, bad);
        if (ncols <= 0) continue;
        k_lub_swap<<<(ncols + LU_THREADS - 1) / LU_THREADS, LU_THREADS, 0, s>>>(g, k0);
        k_lub_u12<<<(ncols + LU_T - 1) / LU_T, LU_THREADS, 0, s>>>(g, k0);
        if (nrows <= 0) continue;
        const int nstrip = (nrows + LU_T - 1) / LU_T;
        const int cw = std::max(LU_T, (ncols + 15) / 16 / LU_T * LU_T + LU_T);   // up to 16 chunks
        const int nchunk = (ncols + cw - 1) / cw;
        k_lub_trail<<<dim3(nstrip, nchunk), LU_THREADS, 0, s>>>(g, k0, cw);
    }
    const int xt = (nown + LU_T - 1) / LU_T;
    for (int k0 = ((n - 1) / LU_P) * LU_P; k0 >= 0; k0 -= LU_P) {
        k_lub_back<<<xt, LU_THREADS, 0, s>>>(g, k0);
        if (k0 > 0) k_lub_back_upd<<<dim3((k0 + LU_T - 1) / LU_T, xt), LU_THREADS, 0, s>>>(g, k0);
    }
    k_lub_extract<<<std::max(nown, 1), LU_THREADS, 0, s>>>(g, c->dbox_ptr, c->dperm, c->dia, c->dja, c->dMinv, ring);
    return cuda_ok(c, cudaGetLastError(), "large-box LU") ? MLF_OK : MLF_E_CUDA;
}

// Every box's rows of the inverse over its neighbourhood: ring null: the near
// list, into c->dMinv (near CSR pattern, allocated by the caller); ring given:
// the 2-ring lists (len[b] unknowns and offset off[b] each, host copies), into
// ring->M2.  *bad_box as mlf_nearinv.
//
// A box's elimination costs ~n^3.  The persistent kernel gives each box one
// CTA, so a box whose work exceeds a few average CTA shares of the rest would
// set the finishing time alone (on the 722-RHS workload's spheroid the
// largest neighbourhoods, 5648 unknowns, took most of the set-up).  Those
// boxes, largest first, run instead on many CTAs each (k_lub_*), on a few side
// streams concurrently with the persistent kernel over the others.
static int blocked_inverse_rows(Ctx* c, int nownmax, const LuRing* ring, const int* ring_len,
                                const long long* ring_off, int* bad_box) {
    DevScope ds;
    const int nb = (int)c->box_ptr.size() - 1;
    int nsm = 0;
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->dev));
    // boxes by decreasing neighbourhood size, so that the largest do not finish last
    auto nsize = [&](int b) { return ring ? ring_len[b] : c->near_ptr[b + 1] - c->near_ptr[b]; };
    std::vector<int> order(nb);
    for (int b = 0; b < nb; ++b) order[b] = b;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b2) { return nsize(a) > nsize(b2); });
    // the large boxes: a prefix of the order, while a box's work exceeds three
    // times the remaining work's share per CTA of the persistent kernel (the
    // many-CTA path serialises each box's panels; measured on the 122 880-RWG
    // spheroid: 128 boxes on it at once the share, 1.79 s; its 32 largest, 1.44 s)
    std::vector<double> tail(nb + 1, 0.0);
    for (int k = nb - 1; k >= 0; --k) tail[k] = tail[k + 1] + std::pow((double)nsize(order[k]), 3.0);
    int nbig = 0;
    while (c->lu_big_min > 0 && nbig < nb && nbig < LU_BIG_MAX && nsize(order[nbig]) >= c->lu_big_min &&
           std::pow((double)nsize(order[nbig]), 3.0) > LU_BIG_FACTOR * tail[nbig] / (2.0 * nsm))
        ++nbig;
    const int nsmall = nb - nbig;
    int *dctr = nullptr, *dbad = nullptr, *dorder = nullptr;
    CK(ds.alloc(&dorder, std::max(nsmall, 1) * sizeof(int)));
    if (nsmall) CK(cudaMemcpyAsync(dorder, order.data() + nbig, nsmall * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    CK(ds.alloc(&dctr, 2 * sizeof(int)));
    dbad = dctr + 1;
    const int init[2] = {0, 0x7fffffff};
    CK(cudaMemcpyAsync(dctr, init, sizeof(init), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    const LuRing none{};
    const LuRing& rg = ring ? *ring : none;
    // large boxes: their own slabs and streams
    const int nstream = std::min(nbig, LU_BIG_STREAMS);
    std::vector<cudaStream_t> bs(nstream, nullptr);
    std::vector<float2*> bslab(nstream, nullptr);
    int* bscr = nullptr;
    int st = MLF_OK;
    if (nbig) {
        const int n0 = nsize(order[0]);
        const size_t bslab_el = (size_t)n0 * n0 + (size_t)n0 * nownmax;
        if (!cuda_ok(c, ds.alloc(&bscr, (size_t)nstream * (LU_P + 1) * sizeof(int)), "large-box scratch"))
            st = MLF_E_CUDA;
        for (int q = 0; q < nstream && !st; ++q)
            if (!cuda_ok(c, ds.alloc(&bslab[q], bslab_el * sizeof(float2)), "large-box slab") ||
                !cuda_ok(c, cudaStreamCreateWithFlags(&bs[q], cudaStreamNonBlocking), "large-box stream"))
                st = MLF_E_CUDA;
    }
    // the persistent kernel over the other boxes: two CTAs per SM, the slabs
    // within half of the free device memory
    if (nsmall && !st) {
        const int ns0 = nsize(order[nbig]);
        const size_t slab = (size_t)ns0 * ns0 + (size_t)ns0 * nownmax;
        size_t fr = 0, tot = 0;
        float2* work = nullptr;
        if (!cuda_ok(c, cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo")) {
            st = MLF_E_CUDA;
        } else {
            const size_t cap = (fr / 2) / (slab * sizeof(float2));
            const int grid = (int)std::max<size_t>(1, std::min<size_t>({(size_t)2 * nsm, (size_t)nsmall, cap}));
            if (!cuda_ok(c, ds.alloc(&work, slab * grid * sizeof(float2)), "neighbourhood LU slabs")) {
                st = MLF_E_CUDA;
            } else {
                k_nbhd_lu32<<<grid, LU_THREADS, 0, c->stream>>>(nsmall, c->dbox_ptr, c->dperm, c->dia, c->dja, c->dZ,
                                                                slab, work, c->dMinv, dorder, dctr, dbad, rg);
                if (!cuda_ok(c, cudaGetLastError(), "neighbourhood LU")) st = MLF_E_CUDA;
            }
        }
    }
    for (int k = 0; k < nbig && !st; ++k) {
        const int q = k % nstream, b = order[k];
        const int n = nsize(b), nown = c->box_ptr[b + 1] - c->box_ptr[b];
        const int* S = ring ? ring->bases + ring_off[b] : c->dja + c->ia[c->box_bases[c->box_ptr[b]]];
        int* scr = bscr + (size_t)q * (LU_P + 1);
        st = big_box_launch(c, rg, b, n, nown, S, bslab[q], scr, scr + LU_P, dbad, bs[q]);
    }
    for (int q = 0; q < nstream; ++q) {
        if (!bs[q]) continue;
        if (!cuda_ok(c, cudaStreamSynchronize(bs[q]), "large-box LU") && !st) st = MLF_E_CUDA;
        cudaStreamDestroy(bs[q]);
    }
    if (st) {
        cudaStreamSynchronize(c->stream);   // the persistent kernel, if launched, ends before its slabs go
        return st;
    }
    int hbad = 0;
    CK(cudaMemcpyAsync(&hbad, dbad, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    *bad_box = hbad == 0x7fffffff ? 0 : hbad;
    c->lu_big_last = nbig;
    return MLF_OK;
}

int nbhd_inverse_lu32(Ctx* c, int nownmax, int* bad_box) {
    return blocked_inverse_rows(c, nownmax, nullptr, nullptr, nullptr, bad_box);
}

int ring_inverse_lu32(Ctx* c, const float2* Zd, const long long* off, const int* len, const int* bases,
                      const std::vector<int>& len_host, const std::vector<long long>& off_host, int nownmax,
                      float2* M2, int* bad_box) {
    LuRing r;
    r.Zd = Zd;
    r.N = c->N;
    r.off = off;
    r.len = len;
    r.bases = bases;
    r.M2 = M2;
    return blocked_inverse_rows(c, nownmax, &r, len_host.data(), off_host.data(), bad_box);
}

}  // namespace mlf

using namespace mlf;

extern "C" int mlf_set_lu_split(mlf_ctx* h, int min_unknowns) {
    if (!h || min_unknowns < 0) return MLF_E_ARG;
    h->c.lu_big_min = min_unknowns;
    return MLF_OK;
}

extern "C" int mlf_get_lu_split(mlf_ctx* h, int* min_unknowns, int* last_big_boxes) {
    if (!h) return MLF_E_ARG;
    if (min_unknowns) *min_unknowns = h->c.lu_big_min;
    if (last_big_boxes) *last_big_boxes = h->c.lu_big_last;
    return MLF_OK;
}
