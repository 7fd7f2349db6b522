// Box-block GEMMs of the FP32 operator on the fifth-generation tensor cores
// (block engine 4): the near field, the leaf aggregation and the leaf receive
// (and the near-pattern preconditioner), as tcgen05.mma with TMEM
// accumulators, operands staged into shared memory by TMA
// (cp.async.bulk.tensor) through tensor maps over this GPU's own memory,
// 3xTF32 for FP32 accuracy.
//
// The near matrix (llenarZesparcida, modMLFMA.f90:1594-1634) is a union of
// dense box-pair blocks Z_ij (bases of leaf box i x bases of near box j).  For
// a block of right-hand sides, leaf box i needs Y_i = sum_j Z_ij X_j.  Here it
// is computed transposed, as a real GEMM whose M side is the right-hand sides:
//   D (2 nrhs x n_i) = A (2 nrhs x 2 n_j) * B^T,   B = [Zr Zi] interleaved
// with the complex product written as a real one on the contraction side:
//   A row 2c   = [ Xr(t,c), -Xi(t,c) ]_t   -> D row 2c   = Re Y(:, c)
//   A row 2c+1 = [ Xi(t,c),  Xr(t,c) ]_t   -> D row 2c+1 = Im Y(:, c)
//   B row p    = [ Zr(p,t),  Zi(p,t) ]_t   (the complex(4) row of Z, as stored)
// so that M = 128 covers 64 right-hand sides exactly and N = the box's bases
// (padded to 16), with no padding of the rows to 128.  The leaf aggregation
// (llenar_campoCyB, modMLFMA.f90:1805-1811: C_b = R_b^T x_b) and receive
// (MatxVec_MLFMA, modMLFMA.f90:1915-1924: y_b = j facy conj(R_b) A_b) are the
// same GEMM with the patterns R in place of Z.
//
// Layouts in HBM (built once per context; the X operand once per call):
//   Z operand: per block e = (i, j) and chunk kc of 16 columns t, the n_i
//     rows p of 32 floats [re, im] x 16 (zero past n_j), rows of all blocks
//     and chunks stacked: one 2-D tensor map [rows][32 floats], boxes of 32
//     rows; split into TF32 hi and lo copies.
//   X operand: per column tile of 64 right-hand sides, per box j and chunk kc,
//     128 rows of 32 floats as above, hi and lo; one tensor map, boxes of 128
//     rows.
//   Aggregation / receive operands: R^T and conj R in the same row format
//     (tc_leaf_setup); the receive's right-hand side operand is the leaf A
//     field itself, read raw.
// Each TMA box of an operand is written with 128-byte swizzling, which is the
// canonical K-major SWIZZLE_128B layout tcgen05.mma reads (8-row atoms of
// 1024 bytes).
//
// A persistent CTA (8 warps) per SM walks work items (tile of at most 160
// rows, 64 columns).  Thread 0 issues the TMA loads of a 3-stage ring; thread
// 32 issues the MMAs: per chunk of 32 real K, 4 K-steps x 3 products (A_lo
// B_hi, A_hi B_lo, A_hi B_hi) into a 128 x N FP32 accumulator in TMEM, and
// tcgen05.commit frees a stage once its MMAs are done.  Warps 4-7 read their
// 32 TMEM lanes each (tcgen05.ld), pair the real and imaginary rows with one
// shuffle and write the output, while the next item accumulates into the
// other of two TMEM accumulators.
//
// Every wait on an mbarrier is bounded; on a timeout the CTA records an error
// flag, lets its loads in flight land, frees its TMEM and skips the output.
// The host checks the flag after the solve (tc_check).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "mlf_internal.h"
#include "mlf_tcgen05.h"

namespace mlf {

#define CK(call)                                             \
    do {                                                     \
        if (!cuda_ok(c, (call), #call)) return MLF_E_CUDA;   \
    } while (0)

constexpr int TC_STAGES = 3;
constexpr int TC_ROWS = 160;                 // bases of box i per tile (MMA N <= 160 here)
constexpr int TC_KCH = 16;                   // complex contraction values per 128-byte TF32 row (receive)
constexpr int TC_KCH_H = 32;                 // complex contraction values per 128-byte FP16 row (near, aggregation)
constexpr int TC_COLS = 64;                  // right-hand sides per column tile (MMA M = 128)
constexpr int TC_ZBOX = 32;                  // rows per TMA box of the Z operand
constexpr int TC_ABYTES = 128 * 128;         // one A tile: 128 rows x 128 bytes
constexpr int TC_BBYTES = TC_ROWS * 128;     // one B tile at most
constexpr int TC_STAGE_BYTES = 2 * TC_ABYTES + 2 * TC_BBYTES;
constexpr size_t TC_SMEM = (size_t)TC_STAGES * TC_STAGE_BYTES + 1024;   // + alignment of the ring
constexpr uint32_t TC_TMEM_COLS = 256;
constexpr uint32_t TC_SPIN = 1u << 20;       // mbarrier polls before a wait gives up

// An operand in rows of 128 bytes: 16 complex values as TF32 (re, im) pairs,
// or 32 as FP16 pairs scaled by a power of two per output row (rinv holds the
// inverse scales), split into hi and lo parts.
struct TcOperand {
    void* hi = nullptr;
    void* lo = nullptr;
    float* rinv = nullptr;
    CUtensorMap mhi, mlo;
};

struct TcState {
    int ntiles = 0, nchunk = 0;     // tiles of the near GEMM; chunks of 32 bases over all boxes
    long long zrows = 0;            // rows of the Z-operand layout
    int nsm = 0;                    // SMs: CTAs of the persistent GEMM
    int4* dtiles = nullptr;         // (box, first row, rows, -), by decreasing work
    int* dtchunks = nullptr;        // per tile: chunks over its near boxes
    int* dzrow = nullptr;           // per block entry e: first Z-operand row (chunk 0)
    int* dcbase = nullptr;          // per box: its first chunk
    int2* dchunk = nullptr;         // per chunk: (first box-sorted position, bases in it)
    int* derr = nullptr;            // set by a CTA whose wait gave up
    unsigned* drowmax = nullptr;    // scratch: per box-sorted basis, the largest magnitude of its near row
    TcOperand Z;
    TcOperand M;                    // the neighbourhood-inverse preconditioner on the near pattern (hi null: not built)
    void *xhi = nullptr, *xlo = nullptr;   // X operand (FP16)
    unsigned* dcmax = nullptr;      // per column: largest magnitude
    float* dcinv = nullptr;         // per column: inverse of its power-of-two scale
    long long xrows_cap = 0;
    int cols_cap = 0;
    CUtensorMap mxhi, mxlo;
    // leaf aggregation and receive (built from the FP32 patterns R on first use)
    const float2* Rsrc = nullptr;   // the patterns the operands below hold
    int K2 = 0;                     // 2K directions of the leaf level
    int natiles = 0;
    int4* datiles = nullptr;        // aggregation tiles (box, first direction, directions, -)
    int* datchunks = nullptr;       // per aggregation tile: chunks of the box's bases
    int* dabase = nullptr;          // per box: first row of the aggregation operand
    int* drbase = nullptr;          // per box: first row of the receive operand
    TcOperand RA;                   // R^T per box and chunk of 32 bases: 2K rows of 32 FP16 (re, im)
    TcOperand RR;                   // conj R per box and chunk of 16 directions: n_b rows of 16 TF32 (re, im)
};

// ---------------------------------------------------------------------------
// operand layouts
// ---------------------------------------------------------------------------

// FP16 scaling: the power of two that takes the largest magnitude m of a row
// (or column) into [2^14, 2^15).  Applying and undoing it is exact; the hi
// part then stays inside the FP16 range and the lo part (2^-11 of it) in its
// normal range for every entry within 2^-14 of m, so the hi/lo split keeps
// the same 22 bits as the TF32 split.
__device__ __forceinline__ int h_scale_exp(float m) {
    if (!(m > 0.f) || !isfinite(m)) return 0;
    int ex;
    frexpf(m, &ex);   // m = f 2^ex, f in [0.5, 1)
    return 15 - ex;
}

__device__ __forceinline__ __half2 h_hi(float a, float b) { return __floats2half2_rn(a, b); }
__device__ __forceinline__ __half2 h_lo(float a, float b, __half2 hi) {
    const float2 h = __half22float2(hi);
    return __floats2half2_rn(a - h.x, b - h.y);
}

// rowmax[i0 + p] = max over the block's row p of |re|, |im| (atomic over the
// near boxes of box i); one CTA per block entry, a thread per row
__global__ void k_blk_rowmax(const int* __restrict__ entry_box, const int* __restrict__ nbox_list,
                             const long long* __restrict__ blk_off, const int* __restrict__ box_ptr,
                             const float2* __restrict__ blk, unsigned* __restrict__ rowmax) {
    const int e = blockIdx.x;
    const int i = entry_box[e], j = nbox_list[e];
    const int i0 = box_ptr[i], ni = box_ptr[i + 1] - i0, nj = box_ptr[j + 1] - box_ptr[j];
    const float2* src = blk + blk_off[e];
    for (int p = threadIdx.x; p < ni; p += blockDim.x) {
        float m = 0.f;
        for (int t = 0; t < nj; ++t) {
            const float2 v = src[(size_t)t * ni + p];
            m = fmaxf(m, fmaxf(fabsf(v.x), fabsf(v.y)));
        }
        atomicMax(rowmax + i0 + p, __float_as_uint(m));
    }
}

__global__ void k_rinv(int n, const unsigned* __restrict__ rowmax, float* __restrict__ rinv) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) rinv[k] = ldexpf(1.f, -h_scale_exp(__uint_as_float(rowmax[k])));
}

// Z operand of block entry e (one CTA each) from the box-pair blocks (column-
// major n_i x n_j at blk_off[e]): row zrow[e] + kc n_i + p holds
// s_p Z(p, 32 kc + u), u = 0..31, as FP16 (re, im) pairs, hi and lo, with
// s_p the power-of-two scale of target basis p's near row.
__global__ void k_tc_fill_zh(const int* __restrict__ entry_box, const int* __restrict__ nbox_list,
                             const long long* __restrict__ blk_off, const int* __restrict__ box_ptr,
                             const int* __restrict__ zrow, const float2* __restrict__ blk,
                             const unsigned* __restrict__ rowmax, __half2* __restrict__ zhi,
                             __half2* __restrict__ zlo) {
    const int e = blockIdx.x;
    const int i = entry_box[e], j = nbox_list[e];
    const int i0 = box_ptr[i], ni = box_ptr[i + 1] - i0, nj = box_ptr[j + 1] - box_ptr[j];
    const int nkc = (nj + TC_KCH_H - 1) / TC_KCH_H;
    const float2* src = blk + blk_off[e];
    const size_t base = (size_t)zrow[e] * TC_KCH_H;
    for (int q = threadIdx.x; q < nkc * ni * TC_KCH_H; q += blockDim.x) {
        const int u = q % TC_KCH_H, rp = q / TC_KCH_H;     // rp = kc n_i + p
        const int kc = rp / ni, p = rp - kc * ni;
        const int t = kc * TC_KCH_H + u;
        const float2 v = t < nj ? src[(size_t)t * ni + p] : make_float2(0.f, 0.f);
        const int ex = h_scale_exp(__uint_as_float(rowmax[i0 + p]));
        const float a = ldexpf(v.x, ex), b = ldexpf(v.y, ex);
        const __half2 h = h_hi(a, b);
        zhi[base + (size_t)rp * TC_KCH_H + u] = h;
        zlo[base + (size_t)rp * TC_KCH_H + u] = h_lo(a, b, h);
    }
}

// cmax[col] = max over column col of xs (box-sorted rows, row-major N x nrhs)
// of |re|, |im|; grid (N / 256, nrhs / 64), 64 columns x 4 row groups per CTA
__global__ void __launch_bounds__(256) k_tc_colmax(int N, int nrhs, const float2* __restrict__ xs,
                                                   unsigned* __restrict__ cmax) {
    __shared__ float red[4][TC_COLS];
    const int tx = threadIdx.x & (TC_COLS - 1), ty = threadIdx.x / TC_COLS;
    const int col = blockIdx.y * TC_COLS + tx;
    const int r0 = blockIdx.x * 256 + ty * 64, r1 = min(r0 + 64, N);
    float m = 0.f;
    if (col < nrhs)
        for (int r = r0; r < r1; ++r) {
            const float2 v = xs[(size_t)r * nrhs + col];
            m = fmaxf(m, fmaxf(fabsf(v.x), fabsf(v.y)));
        }
    red[ty][tx] = m;
    __syncthreads();
    if (ty == 0 && col < nrhs)
        atomicMax(cmax + col, __float_as_uint(fmaxf(fmaxf(red[0][tx], red[1][tx]), fmaxf(red[2][tx], red[3][tx]))));
}

// X operand of one (column tile, chunk of 32 bases) per CTA from xs: rows 2c
// and 2c+1 of the chunk's 128 as in the header, scaled by column c's power of
// two, FP16 hi and lo; cinv receives the inverse scales.
__global__ void __launch_bounds__(256) k_tc_pack_xh(int nchunk, int nrhs, const int2* __restrict__ chunk,
                                                    const float2* __restrict__ xs, const unsigned* __restrict__ cmax,
                                                    __half2* __restrict__ xhi, __half2* __restrict__ xlo,
                                                    float* __restrict__ cinv) {
    __shared__ float2 xsm[TC_KCH_H][TC_COLS + 1];
    __shared__ int sexp[TC_COLS];
    const int ch = blockIdx.x, ct = blockIdx.y;
    const int2 cd = chunk[ch];
    if (threadIdx.x < TC_COLS) {
        const int col = ct * TC_COLS + threadIdx.x;
        const int ex = col < nrhs ? h_scale_exp(__uint_as_float(cmax[col])) : 0;
        sexp[threadIdx.x] = ex;
        if (ch == 0 && col < nrhs) cinv[col] = ldexpf(1.f, -ex);
    }
    for (int q = threadIdx.x; q < TC_KCH_H * TC_COLS; q += blockDim.x) {
        const int u = q / TC_COLS, cl = q - u * TC_COLS, col = ct * TC_COLS + cl;
        xsm[u][cl] = (u < cd.y && col < nrhs) ? xs[(size_t)(cd.x + u) * nrhs + col] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    const size_t base = ((size_t)ct * nchunk + ch) * 128 * TC_KCH_H;
    for (int q = threadIdx.x; q < 128 * TC_KCH_H; q += blockDim.x) {
        const int row = q / TC_KCH_H, u = q - row * TC_KCH_H;
        const float2 v = xsm[u][row >> 1];
        const int ex = sexp[row >> 1];
        const float a = ldexpf((row & 1) ? v.y : v.x, ex), b = ldexpf((row & 1) ? v.x : -v.y, ex);
        const __half2 h = h_hi(a, b);
        xhi[base + (size_t)row * TC_KCH_H + u] = h;
        xlo[base + (size_t)row * TC_KCH_H + u] = h_lo(a, b, h);
    }
}

// Aggregation operand of box b (one CTA per box): row abase[b] + kc 2K + q
// holds s_bq R(32 kc + u, q) for u = 0..31 (zero past the box's bases) as FP16
// hi and lo, s_bq the power-of-two scale of direction q over the box's bases;
// rinv[b 2K + q] = 1 / s_bq.
__global__ void k_tc_fill_rah(int K2, const int* __restrict__ box_ptr, const int* __restrict__ abase,
                              const float2* __restrict__ R, __half2* __restrict__ hi, __half2* __restrict__ lo,
                              float* __restrict__ rinv) {
    const int b = blockIdx.x;
    const int j0 = box_ptr[b], n = box_ptr[b + 1] - j0;
    const int nkc = (n + TC_KCH_H - 1) / TC_KCH_H;
    const size_t base = (size_t)abase[b] * TC_KCH_H;
    for (int q = threadIdx.x; q < K2; q += blockDim.x) {
        float m = 0.f;
        for (int t = 0; t < n; ++t) {
            const float2 v = R[(size_t)(j0 + t) * K2 + q];
            m = fmaxf(m, fmaxf(fabsf(v.x), fabsf(v.y)));
        }
        const int ex = h_scale_exp(m);
        rinv[(size_t)b * K2 + q] = ldexpf(1.f, -ex);
        for (int kc = 0; kc < nkc; ++kc)
            for (int u = 0; u < TC_KCH_H; ++u) {
                const int t = kc * TC_KCH_H + u;
                const float2 v = t < n ? R[(size_t)(j0 + t) * K2 + q] : make_float2(0.f, 0.f);
                const float x = ldexpf(v.x, ex), y = ldexpf(v.y, ex);
                const __half2 h = h_hi(x, y);
                const size_t o = base + ((size_t)kc * K2 + q) * TC_KCH_H + u;
                hi[o] = h;
                lo[o] = h_lo(x, y, h);
            }
    }
}

// Receive operand of box b: row rbase[b] + kc n_b + p holds conj R(p, 16 kc + u)
// for u = 0..15 (zero past the 2K directions).
__global__ void k_tc_fill_rr(int K2, const int* __restrict__ box_ptr, const int* __restrict__ rbase,
                             const float2* __restrict__ R, float* __restrict__ hi, float* __restrict__ lo) {
    const int b = blockIdx.x;
    const int j0 = box_ptr[b], n = box_ptr[b + 1] - j0;
    const int nqc = (K2 + TC_KCH - 1) / TC_KCH;
    const size_t base = (size_t)rbase[b] * 32;
    for (long long e = threadIdx.x; e < (long long)n * nqc * TC_KCH; e += blockDim.x) {
        const int qq = (int)(e % (nqc * TC_KCH));      // 16 kc + u
        const int p = (int)(e / (nqc * TC_KCH));
        const int kc = qq / TC_KCH, u = qq - kc * TC_KCH;
        float2 v = qq < K2 ? R[(size_t)(j0 + p) * K2 + qq] : make_float2(0.f, 0.f);
        v.y = -v.y;
        const float hr = tc::tf32_rna(v.x), hi_ = tc::tf32_rna(v.y);
        const size_t o = base + ((size_t)kc * n + p) * 32 + 2 * u;
        *reinterpret_cast<float2*>(hi + o) = make_float2(hr, hi_);
        *reinterpret_cast<float2*>(lo + o) = make_float2(tc::tf32_rna(v.x - hr), tc::tf32_rna(v.y - hi_));
    }
}

// ---------------------------------------------------------------------------
// the GEMM
// ---------------------------------------------------------------------------

// What one launch computes (B the operand streamed by TMA, X the right-hand
// side operand, tile = (box i, first row r0, rows, instruction descriptor)):
//   TCM_NEAR_ADD  y (FP64 columns, ld) += Z X over the near boxes j of box i
//   TCM_NEAR_SET  out32 (FP32 columns, ld) = M X, M on the near pattern
//   TCM_AGG       C(q, col, i) = sum_t R(t, q) x(t, col), t over box i's bases,
//                 q = r0 .. r0 + rows - 1 of the 2K directions
//   TCM_RECV      y(basis, col) = j facy sum_q conj R(basis, q) A(q, col, i)
// The aggregation takes the near field's packed X operand (the box's own
// chunks); the receive stages raw rows of the A field (64 columns x 16
// directions, 128-byte swizzled) by TMA and warps 2-3 expand them in shared memory
// into the [re, -im] / [im, re] row pairs, split into TF32 hi and lo.
//
// Persistent: one CTA per SM walks the work items q = blockIdx.x + k gridDim.x,
// item q = (tile q / nct, column tile q % nct), the tiles ordered by
// decreasing work.  Warp roles: warp 0 lane 0 issues the TMA loads, warp 1
// lane 0 the MMAs, warps 2-3 expand the receive's raw rows, warps 4-7 read
// the accumulators out (warp 4 + w owns TMEM lanes 32 w .. 32 w + 31).  Two
// TMEM accumulators of 256 columns alternate between items, so the loads and
// MMAs of the next item run under the epilogue of the previous one; the
// shared-memory ring and its barrier phases run on across items.
enum : int { TCM_NEAR_ADD = 0, TCM_NEAR_SET = 1, TCM_AGG = 2, TCM_RECV = 3 };

struct TcArgs {
    const int4* tiles;
    const int* tchunks;  // per tile: chunks of its contraction (near, aggregation)
    int ntiles, nct;     // tiles, column tiles of 64
    const int* box_ptr;
    const int* nbox_ptr;
    const int* nbox_list;
    const int* zrow;     // near: per block entry; aggregation, receive: per box -- first B row
    const int* cbase;    // per box: its first chunk of the X operand
    int nchunk, nrhs, ld, K2;
    float facy;
    const float* rinv;   // FP16 modes: per output row (near: box-sorted basis; aggregation: box x 2K), 1 / scale
    const float* cinv;   // FP16 modes: per column, 1 / scale
    const int* perm;
    double2* y;
    float2* out32;
    float2* C;
    int* err;
};

template <int MODE>
__device__ __forceinline__ int tc_item_chunks(const TcArgs& a, int tile) {
    return MODE == TCM_RECV ? (a.K2 + TC_KCH - 1) / TC_KCH : a.tchunks[tile];
}

// Operands of the near field, its preconditioner and the aggregation are FP16
// (kind::f16, 32 complex values per 128-byte row); the receive's are TF32
// (kind::tf32, 16 per row).  Either way a K step is 32 bytes of the row.
template <int MODE>
struct TcFmt {
    static constexpr bool H = MODE != TCM_RECV;
    static constexpr uint32_t FMT = H ? tc::FMT_F16 : tc::FMT_TF32;
    static constexpr int KCH = H ? TC_KCH_H : TC_KCH;
};

template <int MODE>
__global__ void __launch_bounds__(256, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap mbhi, const __grid_constant__ CUtensorMap mblo,
              const __grid_constant__ CUtensorMap mxhi, const __grid_constant__ CUtensorMap mxlo, const TcArgs a) {
    constexpr bool NEAR = MODE == TCM_NEAR_ADD || MODE == TCM_NEAR_SET;
    constexpr bool RAW = MODE == TCM_RECV;
    constexpr uint32_t RAW_BYTES = TC_COLS * 128;   // 64 field rows of 16 complex values
    extern __shared__ unsigned char tc_raw[];
    __shared__ __align__(8) uint64_t full[TC_STAGES], empty[TC_STAGES], conv[TC_STAGES], accf[2], acce[2], done;
    __shared__ uint32_t tmem_base;
    __shared__ int fail_s, cvok_s, issued_s, consumed_s;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t raw = tc::smem_u32(tc_raw);
    unsigned char* ring = tc_raw + (((raw + 1023u) & ~1023u) - raw);   // 1024-aligned swizzle atoms
    const int nitems = a.ntiles * a.nct;
    volatile int* vfail = &fail_s;
    if (tid == 0) {
        for (int s = 0; s < TC_STAGES; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
            tc::mbar_init(&conv[s], 64);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&accf[b], 1);
            tc::mbar_init(&acce[b], 128);
        }
        tc::mbar_init(&done, 1);
        tc::fence_barrier_init();
        // once any CTA has given up a wait, the rest skip their work (the call fails anyway)
        fail_s = *reinterpret_cast<volatile int*>(a.err) ? 1 : 0;
        issued_s = consumed_s = 0;
    }
    if (warp == 0) {
        tc::tmem_alloc(&tmem_base, 2 * TC_TMEM_COLS);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before_sync();
    __syncthreads();
    tc::tc_fence_after_sync();
    const uint32_t tmem = tmem_base;
    const bool skip_all = fail_s != 0;

    if (warp == 0) {
        if (lane == 0 && !skip_all) {
            // producer: TMA loads of chunk g into stage g % STAGES once that stage's MMAs are done
            tc::tma_prefetch_desc(&mbhi);
            tc::tma_prefetch_desc(&mblo);
            tc::tma_prefetch_desc(&mxhi);
            if (!RAW) tc::tma_prefetch_desc(&mxlo);
            // the B operands stream through once (evicted first from L2); the X
            // operand, read again by the CTAs of every target box near its source
            // box, keeps the normal policy, as does everything after this kernel
            const uint64_t pol_b = tc::l2_evict_first();
            uint32_t g = 0;
            bool ok = true;
            for (int q = blockIdx.x; q < nitems && ok; q += gridDim.x) {
                const int tile = q / a.nct, ct = q - tile * a.nct;
                const int4 tl = a.tiles[tile];
                const int i = tl.x, r0 = tl.y, nrow = tl.z;
                const int ni = a.box_ptr[i + 1] - a.box_ptr[i];
                const int nch = tc_item_chunks<MODE>(a, tile);
                const int nB = (nrow + TC_ZBOX - 1) / TC_ZBOX * TC_ZBOX;          // B rows staged
                const uint32_t bytes = (RAW ? RAW_BYTES : 2u * TC_ABYTES) + 2u * (uint32_t)nB * 128u;
                int le = NEAR ? a.nbox_ptr[i] : 0, lkc = 0;
                for (int cI = 0; cI < nch; ++cI, ++g) {
                    const int s = g % TC_STAGES;
                    if ((g >= TC_STAGES && !tc::mbar_wait(&empty[s], ((g / TC_STAGES) - 1) & 1, TC_SPIN)) || *vfail) {
                        ok = false;   // the consumers then give up on this stage's full barrier too
                        break;
                    }
                    unsigned char* st = ring + (size_t)s * TC_STAGE_BYTES;
                    tc::mbar_arrive_expect_tx(&full[s], bytes);
                    int zr;
                    if (NEAR) {
                        const int j = a.nbox_list[le];
                        const int xr = (ct * a.nchunk + a.cbase[j] + lkc) * 128;
                        tc::tma_load_2d(st, &mxhi, 0, xr, &full[s]);
                        tc::tma_load_2d(st + TC_ABYTES, &mxlo, 0, xr, &full[s]);
                        zr = a.zrow[le] + lkc * ni + r0;
                        if (++lkc * TcFmt<MODE>::KCH >= a.box_ptr[j + 1] - a.box_ptr[j]) {
                            lkc = 0;
                            ++le;
                        }
                    } else if (MODE == TCM_AGG) {
                        const int xr = (ct * a.nchunk + a.cbase[i] + cI) * 128;
                        tc::tma_load_2d(st, &mxhi, 0, xr, &full[s]);
                        tc::tma_load_2d(st + TC_ABYTES, &mxlo, 0, xr, &full[s]);
                        zr = a.zrow[i] + cI * a.K2 + r0;
                    } else {
                        // raw field rows (box i, columns of this tile) into the lo tile's first 8 KB
                        tc::tma_load_2d_hint(st + TC_ABYTES, &mxhi, 2 * TC_KCH * cI, i * a.nrhs + ct * TC_COLS,
                                             &full[s], pol_b);
                        zr = a.zrow[i] + cI * ni + r0;
                    }
                    for (int qq = 0; qq < nB; qq += TC_ZBOX) {
                        // the aggregation's and receive's pattern operands are read by the
                        // tiles of one box (and the column tiles) only: streamed too
                        tc::tma_load_2d_hint(st + 2 * TC_ABYTES + qq * 128, &mbhi, 0, zr + qq, &full[s], pol_b);
                        tc::tma_load_2d_hint(st + 2 * TC_ABYTES + TC_BBYTES + qq * 128, &mblo, 0, zr + qq, &full[s],
                                             pol_b);
                    }
                }
            }
            issued_s = (int)g;
            if (!ok) *vfail = 1;
        }
    } else if (warp == 1) {
        if (lane == 0 && !skip_all) {
            // MMA issuer: per chunk 4 K steps x 3 products into the item's TMEM accumulator
            uint32_t g = 0, na = 0;
            bool ok = true;
            for (int q = blockIdx.x; q < nitems && ok; q += gridDim.x) {
                const int tile = q / a.nct;
                const int nch = tc_item_chunks<MODE>(a, tile);
                if (nch == 0) continue;
                const uint32_t buf = na & 1;
                if (na >= 2 && !tc::mbar_wait(&acce[buf], ((na >> 1) - 1) & 1, TC_SPIN)) {
                    ok = false;
                    break;
                }
                tc::tc_fence_after_sync();
                const uint32_t d = tmem + buf * TC_TMEM_COLS;
                const uint32_t idesc = tc::instr_desc_f32acc(TcFmt<MODE>::FMT, 128, (a.tiles[tile].z + 15) / 16 * 16);
                for (int cI = 0; cI < nch; ++cI, ++g) {
                    const int s = g % TC_STAGES;
                    const uint32_t par = (g / TC_STAGES) & 1;
                    if (!tc::mbar_wait(&full[s], par, TC_SPIN) || (RAW && !tc::mbar_wait(&conv[s], par, TC_SPIN))) {
                        ok = false;
                        break;
                    }
                    tc::tc_fence_after_sync();
                    const uint32_t st = tc::smem_u32(ring + (size_t)s * TC_STAGE_BYTES);
                    const uint32_t ahi = st, alo = st + TC_ABYTES, bhi = st + 2 * TC_ABYTES, blo = bhi + TC_BBYTES;
#pragma unroll
                    for (int k = 0; k < 4; ++k) {   // K steps of 32 bytes of the 128-byte rows
                        const uint32_t ko = 32u * k;
                        const uint64_t dal = tc::kmajor_sw128_desc(alo + ko), dah = tc::kmajor_sw128_desc(ahi + ko);
                        const uint64_t dbl = tc::kmajor_sw128_desc(blo + ko), dbh = tc::kmajor_sw128_desc(bhi + ko);
                        if (TcFmt<MODE>::H) {
                            tc::mma_f16(d, dal, dbh, idesc, (cI | k) != 0);
                            tc::mma_f16(d, dah, dbl, idesc, 1);
                            tc::mma_f16(d, dah, dbh, idesc, 1);
                        } else {
                            tc::mma_tf32(d, dal, dbh, idesc, (cI | k) != 0);
                            tc::mma_tf32(d, dah, dbl, idesc, 1);
                            tc::mma_tf32(d, dah, dbh, idesc, 1);
                        }
                    }
                    tc::mma_commit(&empty[s]);
                }
                if (!ok) break;
                tc::mma_commit(&accf[buf]);   // the item's accumulator is complete
                ++na;
            }
            if (g > 0) {
                tc::mma_commit(&done);   // every MMA issued above
                if (!tc::mbar_wait(&done, 0, TC_SPIN)) ok = false;
            }
            consumed_s = (int)g;
            if (!ok) *vfail = 1;
        }
    } else if (warp < 4) {
        if (RAW && !skip_all) {
            // converters: thread cl expands field row cl (column ct 64 + cl) of each chunk
            const int cl = tid - 64;
            uint32_t g = 0;
            bool go = true;
            for (int q = blockIdx.x; q < nitems && go; q += gridDim.x) {
                const int nch = tc_item_chunks<MODE>(a, q / a.nct);
                for (int cI = 0; cI < nch; ++cI, ++g) {
                    const int s = g % TC_STAGES;
                    const uint32_t par = (g / TC_STAGES) & 1;
                    if (cl == 0) cvok_s = (!*vfail && tc::mbar_wait(&full[s], par, TC_SPIN)) ? 1 : 0;
                    tc::named_bar_sync(1, 64);
                    if (!cvok_s) {   // the same decision in all 64 threads
                        go = false;
                        break;
                    }
                    tc::mbar_wait(&full[s], par, TC_SPIN);   // complete already: acquires the landed bytes
                    unsigned char* st = ring + (size_t)s * TC_STAGE_BYTES;
                    // the raw rows arrive 128-byte swizzled: chunk k of row cl sits at
                    // k ^ (cl & 7), so the 8 lanes of a shared-memory wavefront read 8
                    // different bank groups
                    float4 v[8];
#pragma unroll
                    for (int k = 0; k < 8; ++k)
                        v[k] = *reinterpret_cast<const float4*>(st + TC_ABYTES + tc::sw128_offset(cl, k));
                    tc::named_bar_sync(1, 64);   // every raw row is read before the lo tile overwrites them
                    // rows 2cl and 2cl+1 place chunk k at k ^ (2cl & 7) (resp. +1): lanes
                    // with cl & 4 take the chunks in the order k ^ 1 so that the 8 lanes
                    // of a wavefront again store to 8 different bank groups
                    const int flip = (cl >> 2) & 1;
#pragma unroll
                    for (int kk = 0; kk < 8; ++kk) {   // 16-byte chunk k: complex values 2k, 2k+1
                        const int k = kk ^ flip;
                        const float4 w = flip ? v[kk ^ 1] : v[kk];
                        // row 2cl: (re, -im) pairs; row 2cl+1: (im, re) -- the same values, so
                        // its hi and lo parts follow from row 2cl's (the rounding is symmetric)
                        const float4 eh = make_float4(tc::tf32_rna(w.x), tc::tf32_rna(-w.y), tc::tf32_rna(w.z),
                                                      tc::tf32_rna(-w.w));
                        const float4 el = make_float4(tc::tf32_rna(w.x - eh.x), tc::tf32_rna(-w.y - eh.y),
                                                      tc::tf32_rna(w.z - eh.z), tc::tf32_rna(-w.w - eh.w));
                        const float4 oh = make_float4(-eh.y, eh.x, -eh.w, eh.z);
                        const float4 ol = make_float4(-el.y, el.x, -el.w, el.z);
                        const uint32_t oe = tc::sw128_offset(2 * cl, k), oo = tc::sw128_offset(2 * cl + 1, k);
                        *reinterpret_cast<float4*>(st + oe) = eh;
                        *reinterpret_cast<float4*>(st + oo) = oh;
                        *reinterpret_cast<float4*>(st + TC_ABYTES + oe) = el;
                        *reinterpret_cast<float4*>(st + TC_ABYTES + oo) = ol;
                    }
                    tc::fence_proxy_async_smem();
                    tc::mbar_arrive(&conv[s]);
                }
            }
        }
    } else if (!skip_all) {
        // epilogue: warp 4 + ew reads accumulator rows (TMEM lanes) 32 ew .. 32 ew + 31
        const int ew = warp - 4;
        const int m = 32 * ew + lane;                   // D row = TMEM lane
        uint32_t na = 0;
        for (int q = blockIdx.x; q < nitems; q += gridDim.x) {
            const int tile = q / a.nct, ct = q - tile * a.nct;
            const int4 tl = a.tiles[tile];
            const int i = tl.x, r0 = tl.y, nrow = tl.z;
            const int i0 = a.box_ptr[i];
            const int col = ct * TC_COLS + (m >> 1);
            const bool writer = (lane & 1) == 0 && col < a.nrhs;
            const float cs = (TcFmt<MODE>::H && writer) ? a.cinv[col] : 1.f;
            if (tc_item_chunks<MODE>(a, tile) == 0) {
                // a box without bases radiates nothing
                if (MODE == TCM_AGG && writer)
                    for (int p = 0; p < nrow; ++p) a.C[((size_t)i * a.nrhs + col) * a.K2 + r0 + p] = make_float2(0.f, 0.f);
                continue;
            }
            const uint32_t buf = na & 1;
            // a warp-uniform decision: tcgen05.ld below is a whole-warp instruction
            const bool got = __all_sync(0xffffffffu, tc::mbar_wait(&accf[buf], (na >> 1) & 1, TC_SPIN) ? 1 : 0);
            if (!got) {
                *vfail = 1;
                break;
            }
            tc::tc_fence_after_sync();
            const uint32_t d = tmem + buf * TC_TMEM_COLS + ((uint32_t)(32 * ew) << 16);
            for (int n0 = 0; n0 < nrow; n0 += 32) {
                float v[32];
                tc::tmem_ld_32x32b_x32(d + (uint32_t)n0, v);
#pragma unroll
                for (int u = 0; u < 32; ++u) {
                    const float im = __shfl_xor_sync(0xffffffffu, v[u], 1);
                    const int p = n0 + u;
                    if (writer && p < nrow) {
                        if (MODE == TCM_NEAR_ADD) {
                            const float rs = a.rinv[i0 + r0 + p];   // powers of two: exact
                            double2* yp = a.y + (size_t)col * a.ld + a.perm[i0 + r0 + p];
                            const double2 o = *yp;
                            *yp = make_double2(o.x + (double)(v[u] * rs * cs), o.y + (double)(im * rs * cs));
                        } else if (MODE == TCM_NEAR_SET) {
                            const float rs = a.rinv[i0 + r0 + p];
                            a.out32[(size_t)col * a.ld + a.perm[i0 + r0 + p]] = make_float2(v[u] * rs * cs, im * rs * cs);
                        } else if (MODE == TCM_AGG) {
                            const float rs = a.rinv[(size_t)i * a.K2 + r0 + p];
                            a.C[((size_t)i * a.nrhs + col) * a.K2 + r0 + p] = make_float2(v[u] * rs * cs, im * rs * cs);
                        } else {
                            a.y[(size_t)col * a.ld + a.perm[i0 + r0 + p]] =
                                make_double2(-(double)(a.facy * im), (double)(a.facy * v[u]));
                        }
                    }
                }
            }
            tc::tc_fence_before_sync();
            tc::mbar_arrive(&acce[buf]);   // the MMAs may overwrite this accumulator
            ++na;
        }
    }
    __syncthreads();
    tc::tc_fence_after_sync();
    if (tid == 0 && fail_s) {
        atomicExch(a.err, 1);
        // loads already issued land before the shared memory is given up: at most
        // STAGES chunks beyond the last one the MMA thread consumed
        const uint32_t c0 = (uint32_t)consumed_s, c1 = (uint32_t)issued_s;
        for (uint32_t g = c0; g < c1 && g < c0 + TC_STAGES; ++g)
            tc::mbar_wait(&full[g % TC_STAGES], (g / TC_STAGES) & 1, TC_SPIN);
    }
    tc::tc_fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 2 * TC_TMEM_COLS);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

namespace {

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder(Ctx* c) {
    static std::mutex mu;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::lock_guard<std::mutex> lock(mu);
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !p) {
            c->err = "cuTensorMapEncodeTiled is not available from the driver";
            return nullptr;
        }
        fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// 2-D FP32 tensor map: rows of `inner` floats `row_bytes` apart, boxes of
// box_inner x box_rows, zero fill past the edges
int make_map_2d(Ctx* c, CUtensorMap* m, const void* base, long long inner, long long rows, long long row_bytes,
                int box_inner, int box_rows, CUtensorMapSwizzle swz) {
    auto enc = tensor_map_encoder(c);
    if (!enc) return MLF_E_CUDA;
    const cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)std::max<long long>(rows, 1)};
    const cuuint64_t strides[1] = {(cuuint64_t)row_bytes};
    const cuuint32_t box[2] = {(cuuint32_t)box_inner, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        c->err = "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")";
        return MLF_E_CUDA;
    }
    return MLF_OK;
}

// operand rows of 32 floats (128 bytes), boxes of box_rows rows, 128-byte swizzle
int make_rows_map(Ctx* c, CUtensorMap* m, const void* base, long long rows, int box_rows) {
    return make_map_2d(c, m, base, 32, rows, 128, 32, box_rows, CU_TENSOR_MAP_SWIZZLE_128B);
}

}  // namespace

// tiles in order of decreasing work (chunks), ties in box order: the
// persistent CTAs take them round-robin, longest first
static void order_by_work(std::vector<int4>& tiles, std::vector<int>& nch) {
    std::vector<int> idx(tiles.size());
    for (size_t k = 0; k < idx.size(); ++k) idx[k] = (int)k;
    std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return nch[x] > nch[y]; });
    std::vector<int4> t2(tiles.size());
    std::vector<int> n2(tiles.size());
    for (size_t k = 0; k < idx.size(); ++k) {
        t2[k] = tiles[idx[k]];
        n2[k] = nch[idx[k]];
    }
    tiles.swap(t2);
    nch.swap(n2);
}

void tc_free(Ctx* c) {
    TcState* t = c->tc;
    if (!t) return;
    auto F = [](void* p) { if (p) cudaFree(p); };
    F(t->dtiles); F(t->dzrow); F(t->dcbase); F(t->dchunk); F(t->derr);
    F(t->Z.hi); F(t->Z.lo); F(t->Z.rinv); F(t->M.hi); F(t->M.lo); F(t->M.rinv); F(t->xhi); F(t->xlo);
    F(t->dcmax); F(t->dcinv); F(t->drowmax); F(t->RA.rinv);
    F(t->datiles); F(t->dabase); F(t->drbase); F(t->RA.hi); F(t->RA.lo); F(t->RR.hi); F(t->RR.lo);
    F(t->dtchunks); F(t->datchunks);
    delete t;
    c->tc = nullptr;
}

// FP16 operand of a matrix on the near pattern (the near field Z or the
// preconditioner M) from its box-pair blocks: per-row scales, then the rows
static void tc_operand_free(TcOperand* op) {
    if (op->hi) cudaFree(op->hi);
    if (op->lo) cudaFree(op->lo);
    if (op->rinv) cudaFree(op->rinv);
    op->hi = op->lo = nullptr;
    op->rinv = nullptr;
}

static int tc_near_operand_build(Ctx* c, const float2* blk, TcOperand* op, cudaStream_t s);

// built completely or not at all (a later call would otherwise take a half-built
// operand for a ready one)
static int tc_near_operand(Ctx* c, const float2* blk, TcOperand* op, cudaStream_t s) {
    const int st = tc_near_operand_build(c, blk, op, s);
    if (st) tc_operand_free(op);
    return st;
}

static int tc_near_operand_build(Ctx* c, const float2* blk, TcOperand* op, cudaStream_t s) {
    TcState* t = c->tc;
    const size_t bytes = (size_t)std::max<long long>(t->zrows, 1) * 128;
    CK(cudaMalloc(&op->hi, bytes));
    CK(cudaMalloc(&op->lo, bytes));
    CK(cudaMalloc(&op->rinv, (size_t)std::max(c->N, 1) * sizeof(float)));
    const int ne = (int)c->nbox_list.size();
    CK(cudaMemsetAsync(t->drowmax, 0, (size_t)c->N * sizeof(unsigned), s));
    if (ne) {
        k_blk_rowmax<<<ne, 128, 0, s>>>(c->dblk_entry, c->dnbox_list, c->dblk_off, c->dbox_ptr, blk, t->drowmax);
        k_tc_fill_zh<<<ne, 256, 0, s>>>(c->dblk_entry, c->dnbox_list, c->dblk_off, c->dbox_ptr, t->dzrow, blk,
                                        t->drowmax, static_cast<__half2*>(op->hi), static_cast<__half2*>(op->lo));
    }
    k_rinv<<<(c->N + 255) / 256, 256, 0, s>>>(c->N, t->drowmax, op->rinv);
    CK(cudaGetLastError());
    int st;
    if ((st = make_rows_map(c, &op->mhi, op->hi, t->zrows, TC_ZBOX))) return st;
    if ((st = make_rows_map(c, &op->mlo, op->lo, t->zrows, TC_ZBOX))) return st;
    return MLF_OK;
}

static int tc_setup_build(Ctx* c);

// tiles, chunk tables and the Z operand (needs the box-pair blocks); on a
// failure nothing is kept, so that the next call starts over
static int tc_setup(Ctx* c) {
    if (c->tc) return MLF_OK;
    const int st = tc_setup_build(c);
    if (st) tc_free(c);
    return st;
}

static int tc_setup_build(Ctx* c) {
    int st;
    if ((st = device_blocks_ready(c))) return st;
    const int nb = (int)c->box_ptr.size() - 1;
    const int ne = c->nbox_ptr[nb];
    std::vector<int4> tiles;
    for (int i = 0; i < nb; ++i) {
        const int ni = c->box_ptr[i + 1] - c->box_ptr[i];
        if (ni <= 0) continue;
        const int nt = (ni + TC_ROWS - 1) / TC_ROWS;
        const int per = ((ni + nt - 1) / nt + 15) / 16 * 16;   // rows per tile, multiple of 16
        for (int r0 = 0; r0 < ni; r0 += per) {
            const int nrow = std::min(per, ni - r0);
            if (!tc::valid_shape(128, (nrow + 15) / 16 * 16)) {
                c->err = "tensor-core near field: invalid tile shape";
                return MLF_E_STATE;
            }
            tiles.push_back(make_int4(i, r0, nrow, 0));
        }
    }
    std::vector<int> cbase(nb + 1, 0);
    std::vector<int2> chunk;
    for (int j = 0; j < nb; ++j) {
        const int j0 = c->box_ptr[j], nj = c->box_ptr[j + 1] - j0;
        cbase[j] = (int)chunk.size();
        for (int kc = 0; kc * TC_KCH_H < nj; ++kc)
            chunk.push_back(make_int2(j0 + kc * TC_KCH_H, std::min(TC_KCH_H, nj - kc * TC_KCH_H)));
    }
    cbase[nb] = (int)chunk.size();
    std::vector<int> zrow(std::max(ne, 1), 0);
    long long rows = 0;
    for (int i = 0; i < nb; ++i) {
        const int ni = c->box_ptr[i + 1] - c->box_ptr[i];
        for (int e = c->nbox_ptr[i]; e < c->nbox_ptr[i + 1]; ++e) {
            const int j = c->nbox_list[e];
            zrow[e] = (int)rows;
            rows += (long long)ni * (cbase[j + 1] - cbase[j]);
        }
    }
    if (rows >= (1LL << 31) - 256 || (long long)chunk.size() * 2 * 128 >= (1LL << 31)) {
        c->err = "tensor-core near field: operand layout exceeds 2^31 rows";
        return MLF_E_STATE;
    }
    std::vector<int> tch(tiles.size(), 0);
    for (size_t k = 0; k < tiles.size(); ++k)
        for (int e = c->nbox_ptr[tiles[k].x]; e < c->nbox_ptr[tiles[k].x + 1]; ++e)
            tch[k] += cbase[c->nbox_list[e] + 1] - cbase[c->nbox_list[e]];
    order_by_work(tiles, tch);
    int nsm = 0;
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->dev));
    TcState* t = new TcState();
    t->nsm = std::max(nsm, 1);
    c->tc = t;
    t->ntiles = (int)tiles.size();
    t->nchunk = (int)chunk.size();
    t->zrows = rows;
    CK(cudaMalloc(&t->dtiles, std::max<size_t>(tiles.size(), 1) * sizeof(int4)));
    CK(cudaMalloc(&t->dtchunks, std::max<size_t>(tch.size(), 1) * sizeof(int)));
    CK(cudaMalloc(&t->dzrow, zrow.size() * sizeof(int)));
    CK(cudaMalloc(&t->dcbase, cbase.size() * sizeof(int)));
    CK(cudaMalloc(&t->dchunk, std::max<size_t>(chunk.size(), 1) * sizeof(int2)));
    CK(cudaMalloc(&t->derr, sizeof(int)));
    CK(cudaMalloc(&t->drowmax, std::max(c->N, 1) * sizeof(unsigned)));
    CK(cudaMemcpy(t->dtiles, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(t->dtchunks, tch.data(), tch.size() * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(t->dzrow, zrow.data(), zrow.size() * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(t->dcbase, cbase.data(), cbase.size() * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(t->dchunk, chunk.data(), chunk.size() * sizeof(int2), cudaMemcpyHostToDevice));
    CK(cudaMemset(t->derr, 0, sizeof(int)));
    if ((st = tc_near_operand(c, c->dZblk, &t->Z, c->stream))) return st;
    CK(cudaFuncSetAttribute(k_tc_gemm<TCM_NEAR_ADD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM));
    CK(cudaFuncSetAttribute(k_tc_gemm<TCM_NEAR_SET>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM));
    CK(cudaFuncSetAttribute(k_tc_gemm<TCM_AGG>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM));
    CK(cudaFuncSetAttribute(k_tc_gemm<TCM_RECV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM));
    CK(cudaStreamSynchronize(c->stream));
    return MLF_OK;
}

// X operand buffers for nrhs columns (grown on demand; maps re-encoded)
static int tc_x_buffers(Ctx* c, int nrhs) {
    TcState* t = c->tc;
    const int nct = (nrhs + TC_COLS - 1) / TC_COLS;
    const long long rows = (long long)nct * t->nchunk * 128;
    if (rows <= t->xrows_cap && nct * TC_COLS <= t->cols_cap) return MLF_OK;
    auto F = [](void* p) { if (p) cudaFree(p); };
    F(t->xhi); F(t->xlo); F(t->dcmax); F(t->dcinv);
    t->xhi = t->xlo = nullptr;
    t->dcmax = nullptr;
    t->dcinv = nullptr;
    t->xrows_cap = 0;
    t->cols_cap = 0;
    CK(cudaMalloc(&t->xhi, (size_t)rows * 128));
    CK(cudaMalloc(&t->xlo, (size_t)rows * 128));
    CK(cudaMalloc(&t->dcmax, (size_t)nct * TC_COLS * sizeof(unsigned)));
    CK(cudaMalloc(&t->dcinv, (size_t)nct * TC_COLS * sizeof(float)));
    int st;
    if ((st = make_rows_map(c, &t->mxhi, t->xhi, rows, 128))) return st;
    if ((st = make_rows_map(c, &t->mxlo, t->xlo, rows, 128))) return st;
    t->xrows_cap = rows;
    t->cols_cap = nct * TC_COLS;
    return MLF_OK;
}

// X operand from xs (box-sorted rows, N x nrhs): per-column scales, then the packed FP16 rows
static int tc_pack_x(Ctx* c, const float2* xs, int nrhs, cudaStream_t s) {
    TcState* t = c->tc;
    const int nct = (nrhs + TC_COLS - 1) / TC_COLS;
    CK(cudaMemsetAsync(t->dcmax, 0, (size_t)nrhs * sizeof(unsigned), s));
    k_tc_colmax<<<dim3((c->N + 255) / 256, nct), 256, 0, s>>>(c->N, nrhs, xs, t->dcmax);
    k_tc_pack_xh<<<dim3(t->nchunk, nct), 256, 0, s>>>(t->nchunk, nrhs, t->dchunk, xs, t->dcmax,
                                                      static_cast<__half2*>(t->xhi), static_cast<__half2*>(t->xlo),
                                                      t->dcinv);
    return cuda_ok(c, cudaGetLastError(), "tensor-core X operand") ? MLF_OK : MLF_E_CUDA;
}

// kernel arguments common to every launch
static TcArgs tc_args(const Ctx* c, int nrhs) {
    const TcState* t = c->tc;
    TcArgs a{};
    a.tiles = t->dtiles;
    a.tchunks = t->dtchunks;
    a.ntiles = t->ntiles;
    a.nct = (nrhs + TC_COLS - 1) / TC_COLS;
    a.box_ptr = c->dbox_ptr;
    a.nbox_ptr = c->dnbox_ptr;
    a.nbox_list = c->dnbox_list;
    a.zrow = t->dzrow;
    a.cbase = t->dcbase;
    a.nchunk = t->nchunk;
    a.nrhs = nrhs;
    a.perm = c->dperm;
    a.cinv = t->dcinv;
    a.err = t->derr;
    return a;
}

// persistent grid: one CTA per SM, at most one per work item
static unsigned tc_grid(const TcState* t, const TcArgs& a) {
    return (unsigned)std::max(1, std::min(t->nsm, a.ntiles * a.nct));
}

// y(:, 0:nrhs) += Z_near xs on the tensor cores (engine 4); x_packed: the X
// operand already holds xs (packed by the aggregation of the same product)
int device_near_tc(Ctx* c, const float2* xs, int ld, int nrhs, double2* y, cudaStream_t s, bool x_packed) {
    int st;
    if ((st = tc_setup(c))) return st;
    if ((st = tc_x_buffers(c, nrhs))) return st;
    TcState* t = c->tc;
    if (!x_packed && (st = tc_pack_x(c, xs, nrhs, s))) return st;
    TcArgs a = tc_args(c, nrhs);
    a.ld = ld;
    a.y = y;
    a.rinv = t->Z.rinv;
    k_tc_gemm<TCM_NEAR_ADD><<<tc_grid(t, a), 256, TC_SMEM, s>>>(t->Z.mhi, t->Z.mlo, t->mxhi, t->mxlo, a);
    return cuda_ok(c, cudaGetLastError(), "tensor-core near field") ? MLF_OK : MLF_E_CUDA;
}

// out (FP32 columns, ld N) = M xs for the near-pattern preconditioner M, given
// as box-pair blocks (the layout of the near field's): the same kernel with M
// in place of Z, its operand layout built on first use after each rebuild of M
int device_near_pattern_tc(Ctx* c, const float2* Mblk, const float2* xs, int nrhs, float2* out, cudaStream_t s) {
    int st;
    if ((st = tc_setup(c))) return st;
    if ((st = tc_x_buffers(c, nrhs))) return st;
    TcState* t = c->tc;
    if (!t->M.hi && (st = tc_near_operand(c, Mblk, &t->M, s))) return st;
    if ((st = tc_pack_x(c, xs, nrhs, s))) return st;
    TcArgs a = tc_args(c, nrhs);
    a.ld = c->N;
    a.out32 = out;
    a.rinv = t->M.rinv;
    k_tc_gemm<TCM_NEAR_SET><<<tc_grid(t, a), 256, TC_SMEM, s>>>(t->M.mhi, t->M.mlo, t->mxhi, t->mxlo, a);
    return cuda_ok(c, cudaGetLastError(), "tensor-core near-pattern preconditioner") ? MLF_OK : MLF_E_CUDA;
}

// Aggregation and receive operands of the leaf level from the FP32 patterns R
// (2K values per basis, box-sorted rows), built once per context:
//   RA row abase[b] + kc 2K + q = s_bq R(32 kc + u, q), u = 0..31 (bases of box
//      b), FP16 hi and lo;
//   RR row rbase[b] + kc n_b + p = conj R(p, 16 kc + u), u = 0..15 (directions),
//      TF32 hi and lo;
// zero past the box's bases / the 2K directions.
static int tc_leaf_setup(Ctx* c, const float2* R, int K2) {
    int st;
    if ((st = tc_setup(c))) return st;
    TcState* t = c->tc;
    if (t->RA.hi && t->Rsrc == R && t->K2 == K2) return MLF_OK;
    auto F = [](void* p) { if (p) cudaFree(p); };
    F(t->datiles); F(t->datchunks); F(t->dabase); F(t->drbase);
    F(t->RA.hi); F(t->RA.lo); F(t->RA.rinv); F(t->RR.hi); F(t->RR.lo);
    t->datiles = nullptr; t->datchunks = nullptr; t->dabase = t->drbase = nullptr;
    t->RA.hi = t->RA.lo = t->RR.hi = t->RR.lo = nullptr;
    t->RA.rinv = nullptr;
    t->Rsrc = nullptr;
    const int nb = (int)c->box_ptr.size() - 1;
    const int nqc = (K2 + TC_KCH - 1) / TC_KCH;
    const int nt = (K2 + TC_ROWS - 1) / TC_ROWS;
    const int per = ((K2 + nt - 1) / nt + 15) / 16 * 16;   // directions per tile, multiple of 16, <= 160
    std::vector<int4> tiles;
    std::vector<int> tch;
    std::vector<int> abase(nb + 1, 0), rbase(nb + 1, 0);
    long long arows = 0, rrows = 0;
    for (int b = 0; b < nb; ++b) {
        const int n = c->box_ptr[b + 1] - c->box_ptr[b];
        const int nkc = (n + TC_KCH_H - 1) / TC_KCH_H;
        abase[b] = (int)arows;
        rbase[b] = (int)rrows;
        arows += (long long)nkc * K2;
        rrows += (long long)n * nqc;
        if (arows >= (1LL << 31) - 256 || rrows >= (1LL << 31) - 256) {
            c->err = "tensor-core leaf operators: operand layout exceeds 2^31 rows";
            return MLF_E_STATE;
        }
        for (int r0 = 0; r0 < K2; r0 += per) {
            const int nrow = std::min(per, K2 - r0);
            if (!tc::valid_shape(128, (nrow + 15) / 16 * 16)) {
                c->err = "tensor-core aggregation: invalid tile shape";
                return MLF_E_STATE;
            }
            tiles.push_back(make_int4(b, r0, nrow, 0));
            tch.push_back(nkc);
        }
    }
    order_by_work(tiles, tch);
    abase[nb] = (int)arows;
    rbase[nb] = (int)rrows;
    t->natiles = (int)tiles.size();
    CK(cudaMalloc(&t->datiles, std::max<size_t>(tiles.size(), 1) * sizeof(int4)));
    CK(cudaMalloc(&t->datchunks, std::max<size_t>(tch.size(), 1) * sizeof(int)));
    CK(cudaMalloc(&t->dabase, abase.size() * sizeof(int)));
    CK(cudaMalloc(&t->drbase, rbase.size() * sizeof(int)));
    CK(cudaMemcpy(t->datiles, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(t->datchunks, tch.data(), tch.size() * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(t->dabase, abase.data(), abase.size() * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(t->drbase, rbase.data(), rbase.size() * sizeof(int), cudaMemcpyHostToDevice));
    const size_t ab = (size_t)std::max<long long>(arows, 1) * 128, rb = (size_t)std::max<long long>(rrows, 1) * 128;
    CK(cudaMalloc(&t->RA.hi, ab));
    CK(cudaMalloc(&t->RA.lo, ab));
    CK(cudaMalloc(&t->RA.rinv, (size_t)std::max(nb, 1) * K2 * sizeof(float)));
    CK(cudaMalloc(&t->RR.hi, rb));
    CK(cudaMalloc(&t->RR.lo, rb));
    if (nb) {
        k_tc_fill_rah<<<nb, 256, 0, c->stream>>>(K2, c->dbox_ptr, t->dabase, R, static_cast<__half2*>(t->RA.hi),
                                                 static_cast<__half2*>(t->RA.lo), t->RA.rinv);
        k_tc_fill_rr<<<nb, 256, 0, c->stream>>>(K2, c->dbox_ptr, t->drbase, R, static_cast<float*>(t->RR.hi),
                                                static_cast<float*>(t->RR.lo));
    }
    CK(cudaGetLastError());
    if ((st = make_rows_map(c, &t->RA.mhi, t->RA.hi, arows, TC_ZBOX))) return st;
    if ((st = make_rows_map(c, &t->RA.mlo, t->RA.lo, arows, TC_ZBOX))) return st;
    if ((st = make_rows_map(c, &t->RR.mhi, t->RR.hi, rrows, TC_ZBOX))) return st;
    if ((st = make_rows_map(c, &t->RR.mlo, t->RR.lo, rrows, TC_ZBOX))) return st;
    CK(cudaStreamSynchronize(c->stream));
    t->Rsrc = R;
    t->K2 = K2;
    return MLF_OK;
}

// C (leaf fields, FP32, [box][column][2K]) = R^T xs per box on the tensor
// cores.  Packs the X operand, which the near field of the same product reuses.
int device_agg_tc(Ctx* c, const float2* R, int K, const float2* xs, int nrhs, float2* C, cudaStream_t s) {
    int st;
    if ((st = tc_leaf_setup(c, R, 2 * K))) return st;
    if ((st = tc_x_buffers(c, nrhs))) return st;
    TcState* t = c->tc;
    if ((st = tc_pack_x(c, xs, nrhs, s))) return st;
    TcArgs a = tc_args(c, nrhs);
    a.tiles = t->datiles;
    a.tchunks = t->datchunks;
    a.ntiles = t->natiles;
    a.zrow = t->dabase;
    a.K2 = 2 * K;
    a.C = C;
    a.rinv = t->RA.rinv;
    k_tc_gemm<TCM_AGG><<<tc_grid(t, a), 256, TC_SMEM, s>>>(t->RA.mhi, t->RA.mlo, t->mxhi, t->mxlo, a);
    return cuda_ok(c, cudaGetLastError(), "tensor-core aggregation") ? MLF_OK : MLF_E_CUDA;
}

// y = j facy conj(R) A per leaf box (written, not added) on the tensor cores;
// A the leaf fields [box][column][2K], staged raw by TMA and expanded in the CTA
int device_recv_tc(Ctx* c, const float2* R, int K, const float2* A, float facy, int nrhs, int ld, double2* y,
                   cudaStream_t s) {
    int st;
    const int K2 = 2 * K;
    if ((st = tc_leaf_setup(c, R, K2))) return st;
    TcState* t = c->tc;
    const int nb = (int)c->box_ptr.size() - 1;
    CUtensorMap raw;
    if ((st = make_map_2d(c, &raw, A, 2LL * K2, (long long)nb * nrhs, (long long)K2 * (long long)sizeof(float2),
                          2 * TC_KCH, TC_COLS, CU_TENSOR_MAP_SWIZZLE_128B)))
        return st;
    TcArgs a = tc_args(c, nrhs);
    a.zrow = t->drbase;
    a.K2 = K2;
    a.facy = facy;
    a.ld = ld;
    a.y = y;
    k_tc_gemm<TCM_RECV><<<tc_grid(t, a), 256, TC_SMEM, s>>>(t->RR.mhi, t->RR.mlo, raw, raw, a);
    return cuda_ok(c, cudaGetLastError(), "tensor-core receive") ? MLF_OK : MLF_E_CUDA;
}

// the preconditioner's operand layout is stale once its blocks are rebuilt
void tc_drop_precond(Ctx* c) {
    TcState* t = c->tc;
    if (!t) return;
    tc_operand_free(&t->M);
}

// error flag of the tensor-core kernels since the last check (0: none)
int tc_check(Ctx* c) {
    TcState* t = c->tc;
    if (!t) return MLF_OK;
    int h = 0;
    CK(cudaMemcpy(&h, t->derr, sizeof(int), cudaMemcpyDeviceToHost));
    if (h) {
        CK(cudaMemset(t->derr, 0, sizeof(int)));
        c->err = "tensor-core near field: an mbarrier wait gave up (output skipped)";
        return MLF_E_CUDA;
    }
    return MLF_OK;
}

}  // namespace mlf
