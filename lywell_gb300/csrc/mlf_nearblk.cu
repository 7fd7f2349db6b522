// Near field, leaf aggregation / receive and the own-box preconditioner of the
// FP32 operator for blocks of right-hand sides, as dense per-box complex GEMMs.
//
// The near matrix (llenarZesparcida, modMLFMA.f90:1594-1634) couples every
// basis of a leaf box with every basis of each near leaf box, so its CSR rows
// are unions of whole boxes.  For nrhs > 1 it is applied here as dense
// box-pair blocks: Y_i += Z_ij X_j for each leaf box i and near box j, a
// complex GEMM per pair with X_j (n_j x nrhs) staged in shared memory and each
// Z value read once per tile of right-hand sides.  The CSR form stays the one
// the single-column kernels, ILU and the preconditioners use; the blocks are a
// second copy of the same complex(4) values, built once on first use.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>
#include <type_traits>
#include <unordered_set>
#include <vector>

#include "mlf_internal.h"

namespace mlf {

#define CK(call)                                             \
    do {                                                     \
        if (!cuda_ok(c, (call), #call)) return MLF_E_CUDA;   \
    } while (0)

constexpr int NBK_ROWS = 64;   // rows of box i per CTA
constexpr int NBK_KC = 32;     // source bases per shared-memory chunk

// Zblk[blk_off[e] + t * n_i + p] = Z(perm[box_ptr[i] + p], perm[box_ptr[j] + t])
// for entry e = (i, j); one CTA per entry, the value found by binary search in
// the (column-sorted) CSR row.
__global__ void k_blk_fill(const int* __restrict__ entry_box, const int* __restrict__ nbox_list,
                           const long long* __restrict__ blk_off, const int* __restrict__ box_ptr,
                           const int* __restrict__ perm, const int* __restrict__ ia, const int* __restrict__ ja,
                           const float2* __restrict__ Z, float2* __restrict__ Zblk) {
    const int e = blockIdx.x;
    const int i = entry_box[e], j = nbox_list[e];
    const int i0 = box_ptr[i], ni = box_ptr[i + 1] - i0;
    const int j0 = box_ptr[j], nj = box_ptr[j + 1] - j0;
    float2* out = Zblk + blk_off[e];
    for (int q = threadIdx.x; q < ni * nj; q += blockDim.x) {
        const int t = q / ni, p = q - t * ni;
        const int m = perm[i0 + p], col = perm[j0 + t];
        int lo = ia[m], hi = ia[m + 1] - 1;
        float2 v = make_float2(0.f, 0.f);
        while (lo <= hi) {
            const int mid = (lo + hi) >> 1;
            const int jm = ja[mid];
            if (jm == col) { v = Z[mid]; break; }
            if (jm < col) lo = mid + 1; else hi = mid - 1;
        }
        out[q] = v;
    }
}

// xs[pos * nrhs + r] = x(:, r)[perm[pos]]: box-sorted, row-major copy of the
// input block (FP32 columns or FP64 columns with leading dimension ld)
__global__ void k_blk_pack32(int N, int nrhs, const int* __restrict__ perm, const float2* __restrict__ x32,
                             float2* __restrict__ xs) {
    const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (e >= (size_t)N * nrhs) return;
    const int pos = (int)(e / nrhs), r = (int)(e % nrhs);
    xs[e] = x32[(size_t)r * N + perm[pos]];
}

__global__ void k_blk_pack64(int N, int nrhs, int ld, const int* __restrict__ perm, const double2* __restrict__ x,
                             float2* __restrict__ xs) {
    const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (e >= (size_t)N * nrhs) return;
    const int pos = (int)(e / nrhs), r = (int)(e % nrhs);
    const double2 v = x[(size_t)r * ld + perm[pos]];
    xs[e] = make_float2((float)v.x, (float)v.y);
}

// ---------------------------------------------------------------------------
// Box-block complex GEMM engine.  One CTA (256 threads) computes a 64-row x
// NC = 8 TC column tile of Y = A X for one leaf box, streaming the
// contraction dimension in chunks of 32 through shared memory:
//   A element (row, t): AROW ? A[row * lda + t] : A[t * lda + row] (conj if ACONJ)
//   X element (t, col): XCOL ? X[col * ldx + t] : X[t * ldx + col]
// Two interchangeable multiply engines (the autotuner picks per block size):
//   FmaAcc  FP32 FMAs, thread (ty = tid / 8, tx = tid % 8) owns rows 2 ty,
//           2 ty + 1 and columns TC tx .. TC tx + TC - 1;
//   MmaAcc  tensor-core mma.sync m16n8k8 TF32 with the 3xTF32 split
//           (a_hi b_hi + a_hi b_lo + a_lo b_hi, FP32 accuracy) on the real
//           embedding [Ar Ai] (64 x 64) x [[Br, Bi], [-Bi, Br]] (64 x 2 NC);
//           warp w owns rows 16 (w % 4) .. + 15 and real columns
//           NC (w / 4) .. + NC - 1; the tile is staged through shared memory
//           so the real and imaginary halves meet in one thread.
template <int TC>
struct BlkTile {
    float2 Zs[NBK_KC][NBK_ROWS + 2];
    float2 Xs[NBK_KC][8 * TC];
};

template <int TC>
struct FmaAcc {
    float2 v[2][TC];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int u = 0; u < TC; ++u) v[a][u] = make_float2(0.f, 0.f);
    }
    __device__ __forceinline__ void chunk(const BlkTile<TC>& sm) {
        const int tid = threadIdx.x, ty = tid >> 3, tx = tid & 7;
#pragma unroll 8
        for (int k = 0; k < NBK_KC; ++k) {
            const float4 zz = *reinterpret_cast<const float4*>(&sm.Zs[k][2 * ty]);
#pragma unroll
            for (int u = 0; u < TC; ++u) {
                const float2 xv = sm.Xs[k][tx * TC + u];
                v[0][u].x = fmaf(zz.x, xv.x, v[0][u].x);
                v[0][u].x = fmaf(-zz.y, xv.y, v[0][u].x);
                v[0][u].y = fmaf(zz.x, xv.y, v[0][u].y);
                v[0][u].y = fmaf(zz.y, xv.x, v[0][u].y);
                v[1][u].x = fmaf(zz.z, xv.x, v[1][u].x);
                v[1][u].x = fmaf(-zz.w, xv.y, v[1][u].x);
                v[1][u].y = fmaf(zz.z, xv.y, v[1][u].y);
                v[1][u].y = fmaf(zz.w, xv.x, v[1][u].y);
            }
        }
    }
    // out(row in tile, column in tile, value) for every owned element
    template <class Out>
    __device__ __forceinline__ void store(BlkTile<TC>&, Out out) {
        const int ty = threadIdx.x >> 3, tx = threadIdx.x & 7;
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int u = 0; u < TC; ++u) out(2 * ty + a, tx * TC + u, v[a][u]);
    }
};

__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ void mma_tf32(float (&c)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

template <int TC>
struct MmaAcc {
    float c[TC][4];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int n = 0; n < TC; ++n)
#pragma unroll
            for (int q = 0; q < 4; ++q) c[n][q] = 0.f;
    }
    __device__ __forceinline__ void chunk(const BlkTile<TC>& sm) {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        const int wm = warp & 3, wn = warp >> 2;
        const int g = lane >> 2, t = lane & 3;
        const int r = 16 * wm + g;
#pragma unroll
        for (int ks = 0; ks < 8; ++ks) {
            const bool kim = ks >= 4;              // real k in [32, 64): the imaginary parts of A
            const int kc = (ks & 3) * 8;           // complex k of this step
            const float2 z0 = sm.Zs[kc + t][r], z1 = sm.Zs[kc + t][r + 8];
            const float2 z2 = sm.Zs[kc + t + 4][r], z3 = sm.Zs[kc + t + 4][r + 8];
            const float av[4] = {kim ? z0.y : z0.x, kim ? z1.y : z1.x, kim ? z2.y : z2.x, kim ? z3.y : z3.x};
            uint32_t ah[4], al[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                ah[q] = to_tf32(av[q]);
                al[q] = to_tf32(av[q] - __uint_as_float(ah[q]));
            }
            // B' block: (real rows, real cols) Br, (real rows, imag cols) Bi,
            // (imag rows, real cols) -Bi, (imag rows, imag cols) Br
            const bool use_im = (wn == 0) ? kim : !kim;
            const float sgn = (wn == 0 && kim) ? -1.f : 1.f;
#pragma unroll
            for (int n = 0; n < TC; ++n) {
                const int col = n * 8 + g;
                const float2 x0 = sm.Xs[kc + t][col], x1 = sm.Xs[kc + t + 4][col];
                const float bv[2] = {sgn * (use_im ? x0.y : x0.x), sgn * (use_im ? x1.y : x1.x)};
                uint32_t bh[2], bl[2];
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    bh[q] = to_tf32(bv[q]);
                    bl[q] = to_tf32(bv[q] - __uint_as_float(bh[q]));
                }
                mma_tf32(c[n], al, bh);
                mma_tf32(c[n], ah, bl);
                mma_tf32(c[n], ah, bh);
            }
        }
    }
    template <class Out>
    __device__ __forceinline__ void store(BlkTile<TC>& sm, Out out) {
        constexpr int NC = 8 * TC, LDC = 2 * NC + 1;
        static_assert(sizeof(float) * NBK_ROWS * LDC <= sizeof(BlkTile<TC>), "staging tile");
        float* Cs = reinterpret_cast<float*>(&sm);
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        const int wm = warp & 3, wn = warp >> 2;
        const int g = lane >> 2, t = lane & 3;
        __syncthreads();
#pragma unroll
        for (int n = 0; n < TC; ++n) {
            const int col = wn * NC + n * 8 + 2 * t;
            const int row = 16 * wm + g;
            Cs[row * LDC + col] = c[n][0];
            Cs[row * LDC + col + 1] = c[n][1];
            Cs[(row + 8) * LDC + col] = c[n][2];
            Cs[(row + 8) * LDC + col + 1] = c[n][3];
        }
        __syncthreads();
        for (int e = threadIdx.x; e < NBK_ROWS * NC; e += 256) {
            const int row = e / NC, col = e - row * NC;
            out(row, col, make_float2(Cs[row * LDC + col], Cs[row * LDC + NC + col]));
        }
    }
};

__device__ __forceinline__ void cp_async8(void* dst, const void* src, int src_bytes) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(src), "r"(src_bytes));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

constexpr int NBK_STAGES = 3;

// Y tile += A X over kdim, A and X streamed in chunks of 32 through
// NBK_STAGES cp.async stages (zero-filled past the edges; conjugation of A
// applied by each thread to the values it copied, before the barrier).
template <int TC, bool AROW, bool ACONJ, bool XCOL, class Acc>
__device__ __forceinline__ void blk_mac(Acc& acc, BlkTile<TC>* stage, const float2* __restrict__ A, long long lda,
                                        int r0, int mrows, int kdim, const float2* __restrict__ X, long long ldx,
                                        int c0, int ncols) {
    constexpr int NC = 8 * TC;
    constexpr int ZPT = NBK_KC * NBK_ROWS / 256, XPT = NBK_KC * NC / 256;
    const int tid = threadIdx.x;
    const int nch = (kdim + NBK_KC - 1) / NBK_KC;
    auto zslot = [&](int u, int& k, int& p) {
        const int q = tid + 256 * u;
        if (AROW) { p = q / NBK_KC; k = q - p * NBK_KC; }
        else { k = q / NBK_ROWS; p = q - k * NBK_ROWS; }
    };
    auto issue = [&](int ch) {
        if (ch < nch) {
            BlkTile<TC>& sm = stage[ch % NBK_STAGES];
            const int t0 = ch * NBK_KC;
#pragma unroll
            for (int u = 0; u < ZPT; ++u) {
                int k, p;
                zslot(u, k, p);
                const int t = t0 + k, row = r0 + p;
                const bool ok = t < kdim && row < mrows;
                const float2* src = ok ? (AROW ? A + (size_t)row * lda + t : A + (size_t)t * lda + row) : A;
                cp_async8(&sm.Zs[k][p], src, ok ? 8 : 0);
            }
#pragma unroll
            for (int u = 0; u < XPT; ++u) {
                const int q = tid + 256 * u;
                int k, cc;
                if (XCOL) { cc = q / NBK_KC; k = q - cc * NBK_KC; }
                else { k = q / NC; cc = q - k * NC; }
                const int t = t0 + k, col = c0 + cc;
                const bool ok = t < kdim && col < ncols;
                const float2* src = ok ? (XCOL ? X + (size_t)col * ldx + t : X + (size_t)t * ldx + col) : X;
                cp_async8(&sm.Xs[k][cc], src, ok ? 8 : 0);
            }
        }
        cp_async_commit();
    };
#pragma unroll
    for (int s = 0; s < NBK_STAGES - 1; ++s) issue(s);
    for (int ch = 0; ch < nch; ++ch) {
        cp_async_wait<NBK_STAGES - 2>();
        if (ACONJ) {
            BlkTile<TC>& sm = stage[ch % NBK_STAGES];
#pragma unroll
            for (int u = 0; u < ZPT; ++u) {
                int k, p;
                zslot(u, k, p);
                sm.Zs[k][p].y = -sm.Zs[k][p].y;
            }
        }
        __syncthreads();
        issue(ch + NBK_STAGES - 1);
        acc.chunk(stage[ch % NBK_STAGES]);
    }
    cp_async_wait<0>();
    __syncthreads();
}

// y(:, c0 : c0 + 8 TC) += Z_near x for one 64-row tile of one leaf box.
// The chunks of all near boxes form one sequence, staged through
// NBK_STAGES shared-memory buffers by cp.async (zero-filled past the block
// edges): while chunk c is multiplied, chunks c+1 .. c+STAGES-1 are in flight.
// OUT = 0: y (FP64 columns, ld) += the product; OUT = 1: out32 (FP32 columns,
// ld) = the product (a preconditioner with the near pattern).
template <int TC, class Acc, int OUT>
__global__ void __launch_bounds__(256) k32_near_blk(int nrhs, int ld, const int2* __restrict__ tiles,
                                                    const int* __restrict__ box_ptr, const int* __restrict__ nbox_ptr,
                                                    const int* __restrict__ nbox_list,
                                                    const long long* __restrict__ blk_off,
                                                    const float2* __restrict__ Zblk, const float2* __restrict__ xs,
                                                    const int* __restrict__ perm, double2* __restrict__ y,
                                                    float2* __restrict__ out32) {
    constexpr int NC = 8 * TC;
    constexpr int ZPT = NBK_KC * NBK_ROWS / 256;   // Z values per thread per chunk
    constexpr int XPT = NBK_KC * NC / 256;         // x values per thread per chunk
    extern __shared__ __align__(16) unsigned char near_smem[];
    BlkTile<TC>* stage = reinterpret_cast<BlkTile<TC>*>(near_smem);
    const int2 tl = tiles[blockIdx.x];
    const int i = tl.x, r0 = tl.y, c0 = blockIdx.y * NC;
    const int ni = box_ptr[i + 1] - box_ptr[i];
    const int tid = threadIdx.x;
    const int e_beg = nbox_ptr[i], e_end = nbox_ptr[i + 1];
    int nch = 0;
    for (int e = e_beg; e < e_end; ++e) {
        const int j = nbox_list[e];
        nch += (box_ptr[j + 1] - box_ptr[j] + NBK_KC - 1) / NBK_KC;
    }
    Acc acc;
    acc.zero();
    int le = e_beg, lt = 0;   // next chunk to issue
    auto issue = [&](BlkTile<TC>& sm) {
        if (le < e_end) {
            const int j = nbox_list[le];
            const int j0 = box_ptr[j], nj = box_ptr[j + 1] - j0;
            const float2* zb = Zblk + blk_off[le];
            const float2* xb = xs + (size_t)j0 * nrhs;
#pragma unroll
            for (int u = 0; u < ZPT; ++u) {
                const int q = tid + 256 * u;
                const int k = q / NBK_ROWS, p = q - k * NBK_ROWS;
                const int t = lt + k, row = r0 + p;
                const bool ok = t < nj && row < ni;
                cp_async8(&sm.Zs[k][p], ok ? zb + (size_t)t * ni + row : zb, ok ? 8 : 0);
            }
#pragma unroll
            for (int u = 0; u < XPT; ++u) {
                const int q = tid + 256 * u;
                const int k = q / NC, cc = q - k * NC;
                const int t = lt + k, col = c0 + cc;
                const bool ok = t < nj && col < nrhs;
                cp_async8(&sm.Xs[k][cc], ok ? xb + (size_t)t * nrhs + col : xb, ok ? 8 : 0);
            }
            lt += NBK_KC;
            if (lt >= nj) { ++le; lt = 0; }
        }
        cp_async_commit();   // one group per chunk slot, empty past the end
    };
#pragma unroll
    for (int s = 0; s < NBK_STAGES - 1; ++s) issue(stage[s]);
    for (int cc = 0; cc < nch; ++cc) {
        cp_async_wait<NBK_STAGES - 2>();   // this thread's copies of chunk cc have landed
        __syncthreads();                   // everyone's have; everyone is done with chunk cc-1
        issue(stage[(cc + NBK_STAGES - 1) % NBK_STAGES]);
        acc.chunk(stage[cc % NBK_STAGES]);
    }
    cp_async_wait<0>();
    __syncthreads();
    const int i0 = box_ptr[i];
    acc.store(stage[0], [&](int rt, int ct, float2 v) {
        const int row = r0 + rt, col = c0 + ct;
        if (row < ni && col < nrhs) {
            if (OUT == 0) {
                double2* yp = y + (size_t)col * ld + perm[i0 + row];
                const double2 o = *yp;
                *yp = make_double2(o.x + (double)v.x, o.y + (double)v.y);
            } else {
                out32[(size_t)col * ld + perm[i0 + row]] = v;
            }
        }
    });
}

// Leaf aggregation (llenar_campoCyB step 2, modMLFMA.f90:1805-1811) for a block
// of columns: C(:, col, box) = R_box^T x_box, R_box = the box's 2K x n_b
// patterns.  Grid: (boxes x ceil(2K / 64) row tiles, column tiles).
template <int TC, class Acc>
__global__ void __launch_bounds__(256) k32_agg_blk(int K2, int nrhs, int ntr, const int* __restrict__ box_ptr,
                                                   const float2* __restrict__ R, const float2* __restrict__ xs,
                                                   float2* __restrict__ C) {
    extern __shared__ __align__(16) unsigned char blk_smem[];
    BlkTile<TC>* stage = reinterpret_cast<BlkTile<TC>*>(blk_smem);
    const int b = blockIdx.x / ntr, r0 = (blockIdx.x - b * ntr) * NBK_ROWS, c0 = blockIdx.y * 8 * TC;
    const int j0 = box_ptr[b], nb = box_ptr[b + 1] - j0;
    Acc acc;
    acc.zero();
    blk_mac<TC, false, false, false>(acc, stage, R + (size_t)j0 * K2, K2, r0, K2, nb, xs + (size_t)j0 * nrhs, nrhs,
                                     c0, nrhs);
    acc.store(stage[0], [&](int rt, int ct, float2 v) {
        const int row = r0 + rt, col = c0 + ct;
        if (row < K2 && col < nrhs) C[((size_t)b * nrhs + col) * K2 + row] = v;
    });
}

// Leaf receive (MatxVec_MLFMA, modMLFMA.f90:1915-1924) for a block of
// columns: y(basis, col) = j facy sum_q conj(R[basis][q]) A(q, col, box).
template <int TC, class Acc>
__global__ void __launch_bounds__(256) k32_recv_blk(int K2, int nrhs, int ld, float facy,
                                                    const int2* __restrict__ tiles, const int* __restrict__ box_ptr,
                                                    const int* __restrict__ perm, const float2* __restrict__ R,
                                                    const float2* __restrict__ Af, double2* __restrict__ y) {
    extern __shared__ __align__(16) unsigned char blk_smem[];
    BlkTile<TC>* stage = reinterpret_cast<BlkTile<TC>*>(blk_smem);
    const int2 tl = tiles[blockIdx.x];
    const int b = tl.x, r0 = tl.y, c0 = blockIdx.y * 8 * TC;
    const int j0 = box_ptr[b], nb = box_ptr[b + 1] - j0;
    Acc acc;
    acc.zero();
    blk_mac<TC, true, true, true>(acc, stage, R + (size_t)j0 * K2, K2, r0, nb, K2, Af + (size_t)b * nrhs * K2, K2, c0,
                                  nrhs);
    acc.store(stage[0], [&](int rt, int ct, float2 v) {
        const int row = r0 + rt, col = c0 + ct;
        if (row < nb && col < nrhs)
            y[(size_t)col * ld + perm[j0 + row]] = make_double2(-(double)(facy * v.y), (double)(facy * v.x));
    });
}

// Own-box block preconditioner for a block of FP32 columns:
// out(basis, col) = sum_t M_box[row][t] xs(box basis t, col), M row-major n_b x n_b at boff[box].
template <int TC, class Acc>
__global__ void __launch_bounds__(256) k32_own_blk(int N, int nrhs, const int2* __restrict__ tiles,
                                                   const int* __restrict__ box_ptr, const int* __restrict__ perm,
                                                   const long long* __restrict__ boff, const float2* __restrict__ M,
                                                   const float2* __restrict__ xs, float2* __restrict__ out) {
    extern __shared__ __align__(16) unsigned char blk_smem[];
    BlkTile<TC>* stage = reinterpret_cast<BlkTile<TC>*>(blk_smem);
    const int2 tl = tiles[blockIdx.x];
    const int b = tl.x, r0 = tl.y, c0 = blockIdx.y * 8 * TC;
    const int j0 = box_ptr[b], nb = box_ptr[b + 1] - j0;
    Acc acc;
    acc.zero();
    blk_mac<TC, true, false, false>(acc, stage, M + boff[b], nb, r0, nb, nb, xs + (size_t)j0 * nrhs, nrhs, c0, nrhs);
    acc.store(stage[0], [&](int rt, int ct, float2 v) {
        const int row = r0 + rt, col = c0 + ct;
        if (row < nb && col < nrhs) out[(size_t)col * N + perm[j0 + row]] = v;
    });
}

static int near_blocks_setup(Ctx* c) {
    if (c->blk_ok) return MLF_OK;
    if (need_tree(c)) return MLF_E_STATE;
    const int nb = (int)c->box_ptr.size() - 1;
    if ((int)c->nbox_ptr.size() != nb + 1) {
        c->err = "near box lists missing";
        return MLF_E_STATE;
    }
    const int ne = c->nbox_ptr[nb];
    std::vector<long long> off(ne + 1, 0);
    std::vector<int> entry_box(ne);
    std::vector<int2> tiles;
    for (int i = 0; i < nb; ++i) {
        const int ni = c->box_ptr[i + 1] - c->box_ptr[i];
        for (int e = c->nbox_ptr[i]; e < c->nbox_ptr[i + 1]; ++e) {
            const int j = c->nbox_list[e];
            entry_box[e] = i;
            off[e + 1] = off[e] + (long long)ni * (c->box_ptr[j + 1] - c->box_ptr[j]);
        }
        for (int r0 = 0; r0 < ni; r0 += NBK_ROWS) tiles.push_back(make_int2(i, r0));
    }
    if (off[ne] != c->nnz) {
        c->err = "near blocks do not cover the near CSR";
        return MLF_E_STATE;
    }
    int*& dentry = c->dblk_entry;
    CK(cudaMalloc(&c->dZblk, std::max<long long>(c->nnz, 1) * sizeof(float2)));
    CK(cudaMalloc(&c->dblk_off, (ne + 1) * sizeof(long long)));
    CK(cudaMalloc(&c->dnbox_ptr, (nb + 1) * sizeof(int)));
    CK(cudaMalloc(&c->dnbox_list, std::max(ne, 1) * sizeof(int)));
    CK(cudaMalloc(&c->dblk_tiles, std::max<size_t>(tiles.size(), 1) * sizeof(int2)));
    CK(cudaMalloc(&dentry, std::max(ne, 1) * sizeof(int)));
    CK(cudaMemcpy(c->dblk_off, off.data(), (ne + 1) * sizeof(long long), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->dnbox_ptr, c->nbox_ptr.data(), (nb + 1) * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->dnbox_list, c->nbox_list.data(), ne * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->dblk_tiles, tiles.data(), tiles.size() * sizeof(int2), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dentry, entry_box.data(), ne * sizeof(int), cudaMemcpyHostToDevice));
    if (ne) k_blk_fill<<<ne, 256, 0, c->stream>>>(dentry, c->dnbox_list, c->dblk_off, c->dbox_ptr, c->dperm, c->dia,
                                                  c->dja, c->dZ, c->dZblk);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->stream));
    c->nblk_tiles = (int)tiles.size();
    c->blk_ok = 1;
    return MLF_OK;
}

// dynamic shared memory of the staged kernels: raise each instantiation's
// limit once (before any stream capture)
template <class K>
static size_t staged_smem(K kernel, size_t tile_bytes) {
    const size_t smem = NBK_STAGES * tile_bytes;
    static std::mutex mu;
    static std::unordered_set<const void*> done;   // keyed by the kernel itself
    std::lock_guard<std::mutex> lock(mu);
    if (done.insert((const void*)kernel).second)
        cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return smem;
}

// tile width in columns: the autotuner's choice, else by the block's width
static int blk_width(const Ctx* c, int nrhs) {
    if (c->blk_cols) return c->blk_cols;
    return nrhs <= 8 ? 8 : (nrhs <= 32 ? 32 : 64);
}

// engine x tile width dispatch: F(std::integral_constant<int, TC>, Acc tag)
template <class F>
static void blk_dispatch(const Ctx* c, int nrhs, F f) {
    const int w = blk_width(c, nrhs);
    if (blk_engine_of(c) != 0) {   // the mma.sync engine also stands in for the warp and tensor-core engines
        if (w == 8) f(std::integral_constant<int, 1>(), MmaAcc<1>());
        else if (w == 32) f(std::integral_constant<int, 4>(), MmaAcc<4>());
        else f(std::integral_constant<int, 8>(), MmaAcc<8>());
    } else {
        if (w == 8) f(std::integral_constant<int, 1>(), FmaAcc<1>());
        else if (w == 32) f(std::integral_constant<int, 4>(), FmaAcc<4>());
        else f(std::integral_constant<int, 8>(), FmaAcc<8>());
    }
}

// xs (N x nrhs FP32, box-sorted rows) from FP32 columns (x32, ld N) or FP64 columns (x, ld)
int device_blk_pack(Ctx* c, const double2* x, const float2* x32, int ld, int nrhs, float2* xs, cudaStream_t s) {
    const size_t ne = (size_t)c->N * nrhs;
    if (x32) k_blk_pack32<<<(unsigned)((ne + 255) / 256), 256, 0, s>>>(c->N, nrhs, c->dperm, x32, xs);
    else k_blk_pack64<<<(unsigned)((ne + 255) / 256), 256, 0, s>>>(c->N, nrhs, ld, c->dperm, x, xs);
    return cuda_ok(c, cudaGetLastError(), "pack") ? MLF_OK : MLF_E_CUDA;
}

// y(:, 0:nrhs) += Z_near xs
int device_near_blocks32(Ctx* c, const float2* xs, int ld, int nrhs, double2* y, cudaStream_t s) {
    int st;
    if ((st = near_blocks_setup(c))) return st;
    blk_dispatch(c, nrhs, [&](auto tc, auto acc) {
        constexpr int TC = decltype(tc)::value;
        const size_t smem = staged_smem(k32_near_blk<TC, decltype(acc), 0>, sizeof(BlkTile<TC>));
        k32_near_blk<TC, decltype(acc), 0><<<dim3(c->nblk_tiles, (nrhs + 8 * TC - 1) / (8 * TC)), 256, smem, s>>>(
            nrhs, ld, c->dblk_tiles, c->dbox_ptr, c->dnbox_ptr, c->dnbox_list, c->dblk_off, c->dZblk, xs, c->dperm, y,
            nullptr);
    });
    return cuda_ok(c, cudaGetLastError(), "near blocks") ? MLF_OK : MLF_E_CUDA;
}

// Block copy of a matrix with the near CSR pattern (FP32 values in CSR order)
int device_blocks_from_csr(Ctx* c, const float2* csr, float2** blk) {
    int st;
    if ((st = near_blocks_setup(c))) return st;
    if (!*blk) CK(cudaMalloc(blk, std::max<long long>(c->nnz, 1) * sizeof(float2)));
    const int ne = (int)c->nbox_list.size();
    if (ne) k_blk_fill<<<ne, 256, 0, c->stream>>>(c->dblk_entry, c->dnbox_list, c->dblk_off, c->dbox_ptr, c->dperm,
                                                  c->dia, c->dja, csr, *blk);
    return cuda_ok(c, cudaGetLastError(), "block fill") ? MLF_OK : MLF_E_CUDA;
}

// out (FP32 columns, ld N) = M xs for M given as near-pattern blocks
int device_near_pattern_apply32(Ctx* c, const float2* Mblk, const float2* xs, int nrhs, float2* out, cudaStream_t s) {
    int st;
    if ((st = near_blocks_setup(c))) return st;
    blk_dispatch(c, nrhs, [&](auto tc, auto acc) {
        constexpr int TC = decltype(tc)::value;
        const size_t smem = staged_smem(k32_near_blk<TC, decltype(acc), 1>, sizeof(BlkTile<TC>));
        k32_near_blk<TC, decltype(acc), 1><<<dim3(c->nblk_tiles, (nrhs + 8 * TC - 1) / (8 * TC)), 256, smem, s>>>(
            nrhs, c->N, c->dblk_tiles, c->dbox_ptr, c->dnbox_ptr, c->dnbox_list, c->dblk_off, Mblk, xs, c->dperm,
            nullptr, out);
    });
    return cuda_ok(c, cudaGetLastError(), "near-pattern apply") ? MLF_OK : MLF_E_CUDA;
}

// C (leaf fields, FP32) = R^T x for every leaf box
int device_agg_blocks32(Ctx* c, const float2* R, int K, const float2* xs, int nrhs, float2* C, cudaStream_t s) {
    const int nb = (int)c->box_ptr.size() - 1, K2 = 2 * K, ntr = (K2 + NBK_ROWS - 1) / NBK_ROWS;
    blk_dispatch(c, nrhs, [&](auto tc, auto acc) {
        constexpr int TC = decltype(tc)::value;
        const size_t smem = staged_smem(k32_agg_blk<TC, decltype(acc)>, sizeof(BlkTile<TC>));
        k32_agg_blk<TC, decltype(acc)><<<dim3(nb * ntr, (nrhs + 8 * TC - 1) / (8 * TC)), 256, smem, s>>>(
            K2, nrhs, ntr, c->dbox_ptr, R, xs, C);
    });
    return cuda_ok(c, cudaGetLastError(), "aggregation blocks") ? MLF_OK : MLF_E_CUDA;
}

// y = j facy conj(R) A (leaf receive), written (not added)
int device_recv_blocks32(Ctx* c, const float2* R, int K, const float2* A, float facy, int nrhs, int ld, double2* y,
                         cudaStream_t s) {
    int st;
    if ((st = near_blocks_setup(c))) return st;
    const int K2 = 2 * K;
    blk_dispatch(c, nrhs, [&](auto tc, auto acc) {
        constexpr int TC = decltype(tc)::value;
        const size_t smem = staged_smem(k32_recv_blk<TC, decltype(acc)>, sizeof(BlkTile<TC>));
        k32_recv_blk<TC, decltype(acc)><<<dim3(c->nblk_tiles, (nrhs + 8 * TC - 1) / (8 * TC)), 256, smem, s>>>(
            K2, nrhs, ld, facy, c->dblk_tiles, c->dbox_ptr, c->dperm, R, A, y);
    });
    return cuda_ok(c, cudaGetLastError(), "receive blocks") ? MLF_OK : MLF_E_CUDA;
}

// out (FP32 columns, ld N) = own-box blocks M applied to xs
int device_own_blocks32(Ctx* c, const long long* boff, const float2* M, const float2* xs, int nrhs, float2* out,
                        cudaStream_t s) {
    int st;
    if ((st = near_blocks_setup(c))) return st;
    blk_dispatch(c, nrhs, [&](auto tc, auto acc) {
        constexpr int TC = decltype(tc)::value;
        const size_t smem = staged_smem(k32_own_blk<TC, decltype(acc)>, sizeof(BlkTile<TC>));
        k32_own_blk<TC, decltype(acc)><<<dim3(c->nblk_tiles, (nrhs + 8 * TC - 1) / (8 * TC)), 256, smem, s>>>(
            c->N, nrhs, c->dblk_tiles, c->dbox_ptr, c->dperm, boff, M, xs, out);
    });
    return cuda_ok(c, cudaGetLastError(), "own-box blocks") ? MLF_OK : MLF_E_CUDA;
}

int device_blocks_ready(Ctx* c) { return near_blocks_setup(c); }

void near_blocks_free(Ctx* c) {
    tc_free(c);
    auto F = [](void* p) { if (p) cudaFree(p); };
    F(c->dZblk); F(c->dblk_off); F(c->dnbox_ptr); F(c->dnbox_list); F(c->dblk_tiles); F(c->dblk_entry);
    F(c->dMinvblk);
    warp_engine_free(c);
    c->dZblk = nullptr; c->dblk_off = nullptr; c->dnbox_ptr = nullptr; c->dnbox_list = nullptr;
    c->dblk_tiles = nullptr; c->dblk_entry = nullptr; c->dMinvblk = nullptr;
    c->blk_ok = 0;
}

}  // namespace mlf
