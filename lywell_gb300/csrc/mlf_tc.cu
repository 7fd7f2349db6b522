// Near-field box-pair GEMMs of the FP32 operator on the fifth-generation
// tensor cores (block engine 4): tcgen05.mma with TMEM accumulators, operands
// staged into shared memory by TMA (cp.async.bulk.tensor) through tensor maps
// over this GPU's own memory, 3xTF32 for FP32 accuracy.
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
// (padded to 16), with no padding of the rows to 128.
//
// Layouts in HBM (built once per context; the X operand once per call):
//   Z operand: per block e = (i, j) and chunk kc of 16 columns t, the n_i
//     rows p of 32 floats [re, im] x 16 (zero past n_j), rows of all blocks
//     and chunks stacked: one 2-D tensor map [rows][32 floats], boxes of 32
//     rows; split into TF32 hi and lo copies.
//   X operand: per column tile of 64 right-hand sides, per box j and chunk kc,
//     128 rows of 32 floats as above, hi and lo; one tensor map, boxes of 128
//     rows.
// Each TMA box is written with 128-byte swizzling, which is the canonical
// K-major SWIZZLE_128B layout tcgen05.mma reads (8-row atoms of 1024 bytes).
//
// One CTA (4 warps) per (tile of at most 160 rows of box i, 64 columns).
// Thread 0 (warp 0) issues the TMA loads of a 3-stage ring; thread 32
// (warp 1) issues the MMAs: per chunk of 32 real K, 4 K-steps x 3 products
// (A_lo B_hi, A_hi B_lo, A_hi B_hi) into a 128 x N FP32 accumulator in TMEM,
// and tcgen05.commit frees a stage once its MMAs are done.  The four warps
// then read their 32 TMEM lanes each (tcgen05.ld), pair the real and
// imaginary rows with one shuffle and add into y.
//
// Every wait on an mbarrier is bounded; on a timeout the CTA records an error
// flag, lets its loads in flight land, frees its TMEM and skips the output.
// The host checks the flag after the solve (tc_check).
#include <cuda.h>
#include <cudaTypedefs.h>
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
constexpr int TC_KCH = 16;                   // complex contraction values per chunk (128-byte rows)
constexpr int TC_COLS = 64;                  // right-hand sides per column tile (MMA M = 128)
constexpr int TC_ZBOX = 32;                  // rows per TMA box of the Z operand
constexpr int TC_ABYTES = 128 * 128;         // one A tile: 128 rows x 128 bytes
constexpr int TC_BBYTES = TC_ROWS * 128;     // one B tile at most
constexpr int TC_STAGE_BYTES = 2 * TC_ABYTES + 2 * TC_BBYTES;
constexpr size_t TC_SMEM = (size_t)TC_STAGES * TC_STAGE_BYTES + 1024;   // + alignment of the ring
constexpr uint32_t TC_TMEM_COLS = 256;
constexpr uint32_t TC_SPIN = 1u << 20;       // mbarrier polls before a wait gives up

struct TcOperand {
    float* hi = nullptr;
    float* lo = nullptr;
    CUtensorMap mhi, mlo;
};

struct TcState {
    int ntiles = 0, nchunk = 0;     // tiles of the near GEMM; chunks of 16 bases over all boxes
    long long zrows = 0;            // rows of the Z-operand layout
    int4* dtiles = nullptr;         // (box, first row, rows, instruction descriptor)
    int* dzrow = nullptr;           // per block entry e: first Z-operand row (chunk 0)
    int* dcbase = nullptr;          // per box: its first chunk
    int2* dchunk = nullptr;         // per chunk: (first box-sorted position, bases in it)
    int* derr = nullptr;            // set by a CTA whose wait gave up
    TcOperand Z;
    TcOperand M;                    // the neighbourhood-inverse preconditioner on the near pattern (hi null: not built)
    float *xhi = nullptr, *xlo = nullptr;
    long long xrows_cap = 0;
    CUtensorMap mxhi, mxlo;
    // leaf aggregation and receive (built from the FP32 patterns R on first use)
    const float2* Rsrc = nullptr;   // the patterns the operands below hold
    int K2 = 0;                     // 2K directions of the leaf level
    int natiles = 0;
    int4* datiles = nullptr;        // aggregation tiles (box, first direction, directions, instruction descriptor)
    int* dabase = nullptr;          // per box: first row of the aggregation operand
    int* drbase = nullptr;          // per box: first row of the receive operand
    TcOperand RA;                   // R^T per box and chunk of 16 bases: 2K rows of 16 (re, im)
    TcOperand RR;                   // conj R per box and chunk of 16 directions: n_b rows of 16 (re, im)
};

// ---------------------------------------------------------------------------
// operand layouts
// ---------------------------------------------------------------------------

// Z operand of block entry e (one CTA each) from the box-pair blocks (column-
// major n_i x n_j at blk_off[e]): row zrow[e] + kc n_i + p holds
// Z(p, 16 kc + u), u = 0..15, as (re, im) pairs, split into TF32 hi and lo.
__global__ void k_tc_fill_z(const int* __restrict__ entry_box, const int* __restrict__ nbox_list,
                            const long long* __restrict__ blk_off, const int* __restrict__ box_ptr,
                            const int* __restrict__ zrow, const float2* __restrict__ blk, float* __restrict__ zhi,
                            float* __restrict__ zlo) {
    const int e = blockIdx.x;
    const int i = entry_box[e], j = nbox_list[e];
    const int ni = box_ptr[i + 1] - box_ptr[i], nj = box_ptr[j + 1] - box_ptr[j];
    const int nkc = (nj + TC_KCH - 1) / TC_KCH;
    const float2* src = blk + blk_off[e];
    const size_t base = (size_t)zrow[e] * 32;
    for (int q = threadIdx.x; q < nkc * ni * TC_KCH; q += blockDim.x) {
        const int u = q % TC_KCH, rp = q / TC_KCH;     // rp = kc n_i + p
        const int kc = rp / ni, p = rp - kc * ni;
        const int t = kc * TC_KCH + u;
        const float2 v = t < nj ? src[(size_t)t * ni + p] : make_float2(0.f, 0.f);
        const float hr = tc::tf32_rna(v.x), hi_ = tc::tf32_rna(v.y);
        const size_t o = base + (size_t)rp * 32 + 2 * u;
        zhi[o] = hr;
        zhi[o + 1] = hi_;
        zlo[o] = tc::tf32_rna(v.x - hr);
        zlo[o + 1] = tc::tf32_rna(v.y - hi_);
    }
}

// X operand of one (column tile, chunk) per CTA from xs (box-sorted rows,
// row-major N x nrhs): rows 2c and 2c+1 of the chunk's 128 as in the header.
__global__ void __launch_bounds__(256) k_tc_pack_x(int nchunk, int nrhs, const int2* __restrict__ chunk,
                                                   const float2* __restrict__ xs, float* __restrict__ xhi,
                                                   float* __restrict__ xlo) {
    __shared__ float2 xsm[TC_KCH][TC_COLS + 1];
    const int ch = blockIdx.x, ct = blockIdx.y;
    const int2 cd = chunk[ch];
    for (int q = threadIdx.x; q < TC_KCH * TC_COLS; q += blockDim.x) {
        const int u = q / TC_COLS, cl = q - u * TC_COLS, col = ct * TC_COLS + cl;
        xsm[u][cl] = (u < cd.y && col < nrhs) ? xs[(size_t)(cd.x + u) * nrhs + col] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    const size_t base = ((size_t)ct * nchunk + ch) * 128 * 32;
    for (int q = threadIdx.x; q < 128 * TC_KCH; q += blockDim.x) {
        const int row = q / TC_KCH, u = q - row * TC_KCH;
        const float2 v = xsm[u][row >> 1];
        const float a = (row & 1) ? v.y : v.x, b = (row & 1) ? v.x : -v.y;
        const float ha = tc::tf32_rna(a), hb = tc::tf32_rna(b);
        const size_t o = base + (size_t)row * 32 + 2 * u;
        *reinterpret_cast<float2*>(xhi + o) = make_float2(ha, hb);
        *reinterpret_cast<float2*>(xlo + o) = make_float2(tc::tf32_rna(a - ha), tc::tf32_rna(b - hb));
    }
}

// Aggregation operand of box b (one CTA per box): row abase[b] + kc 2K + q
// holds R(16 kc + u, q) for u = 0..15 (zero past the box's bases).
__global__ void k_tc_fill_ra(int K2, const int* __restrict__ box_ptr, const int* __restrict__ abase,
                             const float2* __restrict__ R, float* __restrict__ hi, float* __restrict__ lo) {
    const int b = blockIdx.x;
    const int j0 = box_ptr[b], n = box_ptr[b + 1] - j0;
    const int nkc = (n + TC_KCH - 1) / TC_KCH;
    const size_t base = (size_t)abase[b] * 32;
    for (long long e = threadIdx.x; e < (long long)nkc * TC_KCH * K2; e += blockDim.x) {
        const int q = (int)(e % K2);
        const int tt = (int)(e / K2);                 // 16 kc + u
        const int kc = tt / TC_KCH, u = tt - kc * TC_KCH;
        const float2 v = tt < n ? R[(size_t)(j0 + tt) * K2 + q] : make_float2(0.f, 0.f);
        const float hr = tc::tf32_rna(v.x), hi_ = tc::tf32_rna(v.y);
        const size_t o = base + ((size_t)kc * K2 + q) * 32 + 2 * u;
        *reinterpret_cast<float2*>(hi + o) = make_float2(hr, hi_);
        *reinterpret_cast<float2*>(lo + o) = make_float2(tc::tf32_rna(v.x - hr), tc::tf32_rna(v.y - hi_));
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
// directions, unswizzled) by TMA and warps 2-3 expand them in shared memory
// into the [re, -im] / [im, re] row pairs, split into TF32 hi and lo.
enum : int { TCM_NEAR_ADD = 0, TCM_NEAR_SET = 1, TCM_AGG = 2, TCM_RECV = 3 };

struct TcArgs {
    const int4* tiles;
    const int* box_ptr;
    const int* nbox_ptr;
    const int* nbox_list;
    const int* zrow;     // near: per block entry; aggregation, receive: per box -- first B row
    const int* cbase;    // per box: its first chunk of the X operand
    int nchunk, nrhs, ld, K2;
    float facy;
    const int* perm;
    double2* y;
    float2* out32;
    float2* C;
    int* err;
};

template <int MODE>
__global__ void __launch_bounds__(128, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap mbhi, const __grid_constant__ CUtensorMap mblo,
              const __grid_constant__ CUtensorMap mxhi, const __grid_constant__ CUtensorMap mxlo, const TcArgs a) {
    constexpr bool NEAR = MODE == TCM_NEAR_ADD || MODE == TCM_NEAR_SET;
    constexpr bool RAW = MODE == TCM_RECV;
    constexpr uint32_t RAW_BYTES = TC_COLS * 128;   // 64 field rows of 16 complex values
    extern __shared__ unsigned char tc_raw[];
    __shared__ __align__(8) uint64_t full[TC_STAGES], empty[TC_STAGES], conv[TC_STAGES], done;
    __shared__ uint32_t tmem_base;
    __shared__ int nch_s, fail_s, cvok_s;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t raw = tc::smem_u32(tc_raw);
    unsigned char* ring = tc_raw + (((raw + 1023u) & ~1023u) - raw);   // 1024-aligned swizzle atoms
    const int4 tl = a.tiles[blockIdx.x];
    const int i = tl.x, r0 = tl.y, nrow = tl.z;
    const uint32_t idesc = (uint32_t)tl.w;
    const int ct = blockIdx.y;
    const int i0 = a.box_ptr[i], ni = a.box_ptr[i + 1] - i0;
    const int e_beg = NEAR ? a.nbox_ptr[i] : 0, e_end = NEAR ? a.nbox_ptr[i + 1] : 0;
    if (tid == 0) {
        for (int s = 0; s < TC_STAGES; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
            tc::mbar_init(&conv[s], 64);
        }
        tc::mbar_init(&done, 1);
        tc::fence_barrier_init();
        int nch = 0;
        if (NEAR) {
            for (int e = e_beg; e < e_end; ++e) {
                const int j = a.nbox_list[e];
                nch += (a.box_ptr[j + 1] - a.box_ptr[j] + TC_KCH - 1) / TC_KCH;
            }
        } else if (MODE == TCM_AGG) {
            nch = (ni + TC_KCH - 1) / TC_KCH;
        } else {
            nch = (a.K2 + TC_KCH - 1) / TC_KCH;
        }
        fail_s = 0;
        // once any CTA has given up a wait, the rest skip their work (the call fails anyway)
        if (*reinterpret_cast<volatile int*>(a.err)) {
            nch = 0;
            fail_s = 1;
        }
        nch_s = nch;
    }
    if (warp == 0) {
        tc::tmem_alloc(&tmem_base, TC_TMEM_COLS);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before_sync();
    __syncthreads();
    tc::tc_fence_after_sync();
    const uint32_t tmem = tmem_base;
    const int nch = nch_s;

    if (tid == 0 && nch > 0) {
        // producer: TMA loads of chunk c into stage c % STAGES once that stage's MMAs are done
        tc::tma_prefetch_desc(&mbhi);
        tc::tma_prefetch_desc(&mblo);
        tc::tma_prefetch_desc(&mxhi);
        if (!RAW) tc::tma_prefetch_desc(&mxlo);
        const int nB = (nrow + TC_ZBOX - 1) / TC_ZBOX * TC_ZBOX;          // B rows staged
        const uint32_t bytes = (RAW ? RAW_BYTES : 2u * TC_ABYTES) + 2u * (uint32_t)nB * 128u;
        int le = e_beg, lkc = 0;
        for (int cI = 0; cI < nch; ++cI) {
            const int s = cI % TC_STAGES;
            if (cI >= TC_STAGES && !tc::mbar_wait(&empty[s], ((cI / TC_STAGES) - 1) & 1, TC_SPIN)) {
                fail_s = 1;   // the consumers then give up on this stage's full barrier too
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
                if (++lkc * TC_KCH >= a.box_ptr[j + 1] - a.box_ptr[j]) {
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
                tc::tma_load_2d(st + TC_ABYTES, &mxhi, 2 * TC_KCH * cI, i * a.nrhs + ct * TC_COLS, &full[s]);
                zr = a.zrow[i] + cI * ni + r0;
            }
            for (int q = 0; q < nB; q += TC_ZBOX) {
                tc::tma_load_2d(st + 2 * TC_ABYTES + q * 128, &mbhi, 0, zr + q, &full[s]);
                tc::tma_load_2d(st + 2 * TC_ABYTES + TC_BBYTES + q * 128, &mblo, 0, zr + q, &full[s]);
            }
        }
    } else if (tid == 32 && nch > 0) {
        // MMA issuer: per chunk 4 K steps x 3 products into the TMEM accumulator
        int consumed = 0;
        bool ok = true;
        for (int cc = 0; cc < nch; ++cc) {
            const int s = cc % TC_STAGES;
            const uint32_t par = (cc / TC_STAGES) & 1;
            if (!tc::mbar_wait(&full[s], par, TC_SPIN) || (RAW && !tc::mbar_wait(&conv[s], par, TC_SPIN))) {
                ok = false;
                break;
            }
            ++consumed;
            tc::tc_fence_after_sync();
            const uint32_t st = tc::smem_u32(ring + (size_t)s * TC_STAGE_BYTES);
            const uint32_t ahi = st, alo = st + TC_ABYTES, bhi = st + 2 * TC_ABYTES, blo = bhi + TC_BBYTES;
#pragma unroll
            for (int q = 0; q < 4; ++q) {   // K steps of 8 TF32 = 32 bytes of the 128-byte rows
                const uint32_t ko = 32u * q;
                tc::mma_tf32(tmem, tc::kmajor_sw128_desc(alo + ko), tc::kmajor_sw128_desc(bhi + ko), idesc,
                             (cc | q) != 0);
                tc::mma_tf32(tmem, tc::kmajor_sw128_desc(ahi + ko), tc::kmajor_sw128_desc(blo + ko), idesc, 1);
                tc::mma_tf32(tmem, tc::kmajor_sw128_desc(ahi + ko), tc::kmajor_sw128_desc(bhi + ko), idesc, 1);
            }
            tc::mma_commit(&empty[s]);
        }
        tc::mma_commit(&done);   // every MMA issued above
        if (!tc::mbar_wait(&done, 0, TC_SPIN)) ok = false;
        if (!ok) {
            // loads already issued land before the shared memory is given up: the
            // producer issues at most STAGES chunks beyond the last one consumed
            for (int k = consumed; k < nch && k < consumed + TC_STAGES; ++k)
                tc::mbar_wait(&full[k % TC_STAGES], (k / TC_STAGES) & 1, TC_SPIN);
            fail_s = 1;
        }
    } else if (RAW && tid >= 64 && nch > 0) {
        // converters: thread c expands field row c (column ct 64 + c) of each chunk
        const int cl = tid - 64;
        for (int cc = 0; cc < nch; ++cc) {
            const int s = cc % TC_STAGES;
            const uint32_t par = (cc / TC_STAGES) & 1;
            if (cl == 0) cvok_s = tc::mbar_wait(&full[s], par, TC_SPIN) ? 1 : 0;
            tc::named_bar_sync(1, 64);
            if (!cvok_s) break;   // the same decision in all 64 threads
            tc::mbar_wait(&full[s], par, TC_SPIN);   // complete already: acquires the landed bytes
            unsigned char* st = ring + (size_t)s * TC_STAGE_BYTES;
            const float4* src = reinterpret_cast<const float4*>(st + TC_ABYTES + cl * 128);
            float4 v[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) v[q] = src[q];
            tc::named_bar_sync(1, 64);   // every raw row is read before the lo tile overwrites them
#pragma unroll
            for (int q = 0; q < 8; ++q) {   // 16-byte chunk q: complex values 2q, 2q+1
                const float4 w = v[q];
                const float4 ev = make_float4(w.x, -w.y, w.z, -w.w), od = make_float4(w.y, w.x, w.w, w.z);
                const float4 eh = make_float4(tc::tf32_rna(ev.x), tc::tf32_rna(ev.y), tc::tf32_rna(ev.z),
                                              tc::tf32_rna(ev.w));
                const float4 oh = make_float4(tc::tf32_rna(od.x), tc::tf32_rna(od.y), tc::tf32_rna(od.z),
                                              tc::tf32_rna(od.w));
                const float4 el = make_float4(tc::tf32_rna(ev.x - eh.x), tc::tf32_rna(ev.y - eh.y),
                                              tc::tf32_rna(ev.z - eh.z), tc::tf32_rna(ev.w - eh.w));
                const float4 ol = make_float4(tc::tf32_rna(od.x - oh.x), tc::tf32_rna(od.y - oh.y),
                                              tc::tf32_rna(od.z - oh.z), tc::tf32_rna(od.w - oh.w));
                const uint32_t oe = tc::sw128_offset(2 * cl, q), oo = tc::sw128_offset(2 * cl + 1, q);
                *reinterpret_cast<float4*>(st + oe) = eh;
                *reinterpret_cast<float4*>(st + oo) = oh;
                *reinterpret_cast<float4*>(st + TC_ABYTES + oe) = el;
                *reinterpret_cast<float4*>(st + TC_ABYTES + oo) = ol;
            }
            tc::fence_proxy_async_smem();
            tc::mbar_arrive(&conv[s]);
        }
    }
    __syncthreads();
    tc::tc_fence_after_sync();
    if (tid == 0 && fail_s) atomicExch(a.err, 1);
    if (fail_s == 0 && nch > 0) {
        const int m = 32 * warp + lane;                 // D row = TMEM lane
        const int col = ct * TC_COLS + (m >> 1);
        const bool writer = (lane & 1) == 0 && col < a.nrhs;
        for (int n0 = 0; n0 < nrow; n0 += 32) {
            float v[32];
            tc::tmem_ld_32x32b_x32(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)n0, v);
#pragma unroll
            for (int u = 0; u < 32; ++u) {
                const float im = __shfl_xor_sync(0xffffffffu, v[u], 1);
                const int p = n0 + u;
                if (writer && p < nrow) {
                    if (MODE == TCM_NEAR_ADD) {
                        double2* yp = a.y + (size_t)col * a.ld + a.perm[i0 + r0 + p];
                        const double2 o = *yp;
                        *yp = make_double2(o.x + (double)v[u], o.y + (double)im);
                    } else if (MODE == TCM_NEAR_SET) {
                        a.out32[(size_t)col * a.ld + a.perm[i0 + r0 + p]] = make_float2(v[u], im);
                    } else if (MODE == TCM_AGG) {
                        a.C[((size_t)i * a.nrhs + col) * a.K2 + r0 + p] = make_float2(v[u], im);
                    } else {
                        a.y[(size_t)col * a.ld + a.perm[i0 + r0 + p]] =
                            make_double2(-(double)(a.facy * im), (double)(a.facy * v[u]));
                    }
                }
            }
        }
    } else if (MODE == TCM_AGG && fail_s == 0) {
        // a box without bases radiates nothing
        const int m = 32 * warp + lane;
        const int col = ct * TC_COLS + (m >> 1);
        if ((lane & 1) == 0 && col < a.nrhs)
            for (int p = 0; p < nrow; ++p) a.C[((size_t)i * a.nrhs + col) * a.K2 + r0 + p] = make_float2(0.f, 0.f);
    }
    tc::tc_fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, TC_TMEM_COLS);
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
int make_map_2d(Ctx* c, CUtensorMap* m, const float* base, long long inner, long long rows, long long row_bytes,
                int box_inner, int box_rows, CUtensorMapSwizzle swz) {
    auto enc = tensor_map_encoder(c);
    if (!enc) return MLF_E_CUDA;
    const cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)std::max<long long>(rows, 1)};
    const cuuint64_t strides[1] = {(cuuint64_t)row_bytes};
    const cuuint32_t box[2] = {(cuuint32_t)box_inner, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        c->err = "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")";
        return MLF_E_CUDA;
    }
    return MLF_OK;
}

// operand rows of 32 floats (128 bytes), boxes of box_rows rows, 128-byte swizzle
int make_rows_map(Ctx* c, CUtensorMap* m, const float* base, long long rows, int box_rows) {
    return make_map_2d(c, m, base, 32, rows, 128, 32, box_rows, CU_TENSOR_MAP_SWIZZLE_128B);
}

}  // namespace

void tc_free(Ctx* c) {
    TcState* t = c->tc;
    if (!t) return;
    auto F = [](void* p) { if (p) cudaFree(p); };
    F(t->dtiles); F(t->dzrow); F(t->dcbase); F(t->dchunk); F(t->derr);
    F(t->Z.hi); F(t->Z.lo); F(t->M.hi); F(t->M.lo); F(t->xhi); F(t->xlo);
    F(t->datiles); F(t->dabase); F(t->drbase); F(t->RA.hi); F(t->RA.lo); F(t->RR.hi); F(t->RR.lo);
    delete t;
    c->tc = nullptr;
}

// tiles, chunk tables and the Z operand (needs the box-pair blocks)
static int tc_setup(Ctx* c) {
    if (c->tc) return MLF_OK;
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
            const int N = (nrow + 15) / 16 * 16;
            if (!tc::valid_shape(128, N)) {
                c->err = "tensor-core near field: invalid tile shape";
                return MLF_E_STATE;
            }
            tiles.push_back(make_int4(i, r0, nrow, (int)tc::instr_desc_f32acc(tc::FMT_TF32, 128, N)));
        }
    }
    std::vector<int> cbase(nb + 1, 0);
    std::vector<int2> chunk;
    for (int j = 0; j < nb; ++j) {
        const int j0 = c->box_ptr[j], nj = c->box_ptr[j + 1] - j0;
        cbase[j] = (int)chunk.size();
        for (int kc = 0; kc * TC_KCH < nj; ++kc) chunk.push_back(make_int2(j0 + kc * TC_KCH, std::min(TC_KCH, nj - kc * TC_KCH)));
    }
    cbase[nb] = (int)chunk.size();
    std::vector<int> zrow(std::max(ne, 1), 0);
    long long rows = 0;
    for (int i = 0; i < nb; ++i) {
        const int ni = c->box_ptr[i + 1] - c->box_ptr[i];
        for (int e = c->nbox_ptr[i]; e < c->nbox_ptr[i + 1]; ++e) {
            const int j = c->nbox_list[e];
            zrow[e] = (int)rows;
            rows += (long long)ni * ((c->box_ptr[j + 1] - c->box_ptr[j] + TC_KCH - 1) / TC_KCH);
        }
    }
    if (rows >= (1LL << 31) - 256 || (long long)chunk.size() * 2 * 128 >= (1LL << 31)) {
        c->err = "tensor-core near field: operand layout exceeds 2^31 rows";
        return MLF_E_STATE;
    }
    TcState* t = new TcState();
    c->tc = t;
    t->ntiles = (int)tiles.size();
    t->nchunk = (int)chunk.size();
    t->zrows = rows;
    CK(cudaMalloc(&t->dtiles, std::max<size_t>(tiles.size(), 1) * sizeof(int4)));
    CK(cudaMalloc(&t->dzrow, zrow.size() * sizeof(int)));
    CK(cudaMalloc(&t->dcbase, cbase.size() * sizeof(int)));
    CK(cudaMalloc(&t->dchunk, std::max<size_t>(chunk.size(), 1) * sizeof(int2)));
    CK(cudaMalloc(&t->derr, sizeof(int)));
    CK(cudaMemcpy(t->dtiles, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(t->dzrow, zrow.data(), zrow.size() * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(t->dcbase, cbase.data(), cbase.size() * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(t->dchunk, chunk.data(), chunk.size() * sizeof(int2), cudaMemcpyHostToDevice));
    CK(cudaMemset(t->derr, 0, sizeof(int)));
    const size_t zfl = (size_t)std::max<long long>(rows, 1) * 32;
    CK(cudaMalloc(&t->Z.hi, zfl * sizeof(float)));
    CK(cudaMalloc(&t->Z.lo, zfl * sizeof(float)));
    if (ne)
        k_tc_fill_z<<<ne, 256, 0, c->stream>>>(c->dblk_entry, c->dnbox_list, c->dblk_off, c->dbox_ptr, t->dzrow,
                                               c->dZblk, t->Z.hi, t->Z.lo);
    CK(cudaGetLastError());
    if ((st = make_rows_map(c, &t->Z.mhi, t->Z.hi, rows, TC_ZBOX))) return st;
    if ((st = make_rows_map(c, &t->Z.mlo, t->Z.lo, rows, TC_ZBOX))) return st;
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
    if (rows <= t->xrows_cap) return MLF_OK;
    if (t->xhi) cudaFree(t->xhi);
    if (t->xlo) cudaFree(t->xlo);
    t->xhi = t->xlo = nullptr;
    t->xrows_cap = 0;
    CK(cudaMalloc(&t->xhi, (size_t)rows * 32 * sizeof(float)));
    CK(cudaMalloc(&t->xlo, (size_t)rows * 32 * sizeof(float)));
    int st;
    if ((st = make_rows_map(c, &t->mxhi, t->xhi, rows, 128))) return st;
    if ((st = make_rows_map(c, &t->mxlo, t->xlo, rows, 128))) return st;
    t->xrows_cap = rows;
    return MLF_OK;
}

// kernel arguments common to every launch
static TcArgs tc_args(const Ctx* c, int nrhs) {
    const TcState* t = c->tc;
    TcArgs a{};
    a.tiles = t->dtiles;
    a.box_ptr = c->dbox_ptr;
    a.nbox_ptr = c->dnbox_ptr;
    a.nbox_list = c->dnbox_list;
    a.zrow = t->dzrow;
    a.cbase = t->dcbase;
    a.nchunk = t->nchunk;
    a.nrhs = nrhs;
    a.perm = c->dperm;
    a.err = t->derr;
    return a;
}

// y(:, 0:nrhs) += Z_near xs on the tensor cores (engine 4); x_packed: the X
// operand already holds xs (packed by the aggregation of the same product)
int device_near_tc(Ctx* c, const float2* xs, int ld, int nrhs, double2* y, cudaStream_t s, bool x_packed) {
    int st;
    if ((st = tc_setup(c))) return st;
    if ((st = tc_x_buffers(c, nrhs))) return st;
    TcState* t = c->tc;
    const int nct = (nrhs + TC_COLS - 1) / TC_COLS;
    if (!x_packed) k_tc_pack_x<<<dim3(t->nchunk, nct), 256, 0, s>>>(t->nchunk, nrhs, t->dchunk, xs, t->xhi, t->xlo);
    TcArgs a = tc_args(c, nrhs);
    a.ld = ld;
    a.y = y;
    k_tc_gemm<TCM_NEAR_ADD><<<dim3(t->ntiles, nct), 128, TC_SMEM, s>>>(t->Z.mhi, t->Z.mlo, t->mxhi, t->mxlo, a);
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
    if (!t->M.hi) {
        const size_t zfl = (size_t)std::max<long long>(t->zrows, 1) * 32;
        CK(cudaMalloc(&t->M.hi, zfl * sizeof(float)));
        CK(cudaMalloc(&t->M.lo, zfl * sizeof(float)));
        const int ne = (int)c->nbox_list.size();
        if (ne)
            k_tc_fill_z<<<ne, 256, 0, s>>>(c->dblk_entry, c->dnbox_list, c->dblk_off, c->dbox_ptr, t->dzrow, Mblk,
                                           t->M.hi, t->M.lo);
        CK(cudaGetLastError());
        if ((st = make_rows_map(c, &t->M.mhi, t->M.hi, t->zrows, TC_ZBOX))) return st;
        if ((st = make_rows_map(c, &t->M.mlo, t->M.lo, t->zrows, TC_ZBOX))) return st;
    }
    const int nct = (nrhs + TC_COLS - 1) / TC_COLS;
    k_tc_pack_x<<<dim3(t->nchunk, nct), 256, 0, s>>>(t->nchunk, nrhs, t->dchunk, xs, t->xhi, t->xlo);
    TcArgs a = tc_args(c, nrhs);
    a.ld = c->N;
    a.out32 = out;
    k_tc_gemm<TCM_NEAR_SET><<<dim3(t->ntiles, nct), 128, TC_SMEM, s>>>(t->M.mhi, t->M.mlo, t->mxhi, t->mxlo, a);
    return cuda_ok(c, cudaGetLastError(), "tensor-core near-pattern preconditioner") ? MLF_OK : MLF_E_CUDA;
}

// Aggregation and receive operands of the leaf level from the FP32 patterns R
// (2K values per basis, box-sorted rows), built once per context:
//   RA row abase[b] + kc 2K + q = R(16 kc + u, q), u = 0..15 (bases of box b),
//   RR row rbase[b] + kc n_b + p = conj R(p, 16 kc + u), u = 0..15 (directions),
// zero past the box's bases / the 2K directions, split into TF32 hi and lo.
static int tc_leaf_setup(Ctx* c, const float2* R, int K2) {
    int st;
    if ((st = tc_setup(c))) return st;
    TcState* t = c->tc;
    if (t->RA.hi && t->Rsrc == R && t->K2 == K2) return MLF_OK;
    auto F = [](void* p) { if (p) cudaFree(p); };
    F(t->datiles); F(t->dabase); F(t->drbase); F(t->RA.hi); F(t->RA.lo); F(t->RR.hi); F(t->RR.lo);
    t->datiles = nullptr; t->dabase = t->drbase = nullptr;
    t->RA.hi = t->RA.lo = t->RR.hi = t->RR.lo = nullptr;
    t->Rsrc = nullptr;
    const int nb = (int)c->box_ptr.size() - 1;
    const int nqc = (K2 + TC_KCH - 1) / TC_KCH;
    const int nt = (K2 + TC_ROWS - 1) / TC_ROWS;
    const int per = ((K2 + nt - 1) / nt + 15) / 16 * 16;   // directions per tile, multiple of 16, <= 160
    std::vector<int4> tiles;
    std::vector<int> abase(nb + 1, 0), rbase(nb + 1, 0);
    long long arows = 0, rrows = 0;
    for (int b = 0; b < nb; ++b) {
        const int n = c->box_ptr[b + 1] - c->box_ptr[b];
        abase[b] = (int)arows;
        rbase[b] = (int)rrows;
        arows += (long long)((n + TC_KCH - 1) / TC_KCH) * K2;
        rrows += (long long)n * nqc;
        if (arows >= (1LL << 31) - 256 || rrows >= (1LL << 31) - 256) {
            c->err = "tensor-core leaf operators: operand layout exceeds 2^31 rows";
            return MLF_E_STATE;
        }
        for (int r0 = 0; r0 < K2; r0 += per) {
            const int nrow = std::min(per, K2 - r0);
            const int N = (nrow + 15) / 16 * 16;
            if (!tc::valid_shape(128, N)) {
                c->err = "tensor-core aggregation: invalid tile shape";
                return MLF_E_STATE;
            }
            tiles.push_back(make_int4(b, r0, nrow, (int)tc::instr_desc_f32acc(tc::FMT_TF32, 128, N)));
        }
    }
    abase[nb] = (int)arows;
    rbase[nb] = (int)rrows;
    t->natiles = (int)tiles.size();
    CK(cudaMalloc(&t->datiles, std::max<size_t>(tiles.size(), 1) * sizeof(int4)));
    CK(cudaMalloc(&t->dabase, abase.size() * sizeof(int)));
    CK(cudaMalloc(&t->drbase, rbase.size() * sizeof(int)));
    CK(cudaMemcpy(t->datiles, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(t->dabase, abase.data(), abase.size() * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(t->drbase, rbase.data(), rbase.size() * sizeof(int), cudaMemcpyHostToDevice));
    const size_t afl = (size_t)std::max<long long>(arows, 1) * 32, rfl = (size_t)std::max<long long>(rrows, 1) * 32;
    CK(cudaMalloc(&t->RA.hi, afl * sizeof(float)));
    CK(cudaMalloc(&t->RA.lo, afl * sizeof(float)));
    CK(cudaMalloc(&t->RR.hi, rfl * sizeof(float)));
    CK(cudaMalloc(&t->RR.lo, rfl * sizeof(float)));
    if (nb) {
        k_tc_fill_ra<<<nb, 256, 0, c->stream>>>(K2, c->dbox_ptr, t->dabase, R, t->RA.hi, t->RA.lo);
        k_tc_fill_rr<<<nb, 256, 0, c->stream>>>(K2, c->dbox_ptr, t->drbase, R, t->RR.hi, t->RR.lo);
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
    const int nct = (nrhs + TC_COLS - 1) / TC_COLS;
    k_tc_pack_x<<<dim3(t->nchunk, nct), 256, 0, s>>>(t->nchunk, nrhs, t->dchunk, xs, t->xhi, t->xlo);
    TcArgs a = tc_args(c, nrhs);
    a.tiles = t->datiles;
    a.zrow = t->dabase;
    a.K2 = 2 * K;
    a.C = C;
    k_tc_gemm<TCM_AGG><<<dim3(t->natiles, nct), 128, TC_SMEM, s>>>(t->RA.mhi, t->RA.mlo, t->mxhi, t->mxlo, a);
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
    if ((st = make_map_2d(c, &raw, reinterpret_cast<const float*>(A), 2LL * K2, (long long)nb * nrhs,
                          (long long)K2 * (long long)sizeof(float2), 2 * TC_KCH, TC_COLS, CU_TENSOR_MAP_SWIZZLE_NONE)))
        return st;
    const int nct = (nrhs + TC_COLS - 1) / TC_COLS;
    TcArgs a = tc_args(c, nrhs);
    a.zrow = t->drbase;
    a.K2 = K2;
    a.facy = facy;
    a.ld = ld;
    a.y = y;
    k_tc_gemm<TCM_RECV><<<dim3(t->ntiles, nct), 128, TC_SMEM, s>>>(t->RR.mhi, t->RR.mlo, raw, raw, a);
    return cuda_ok(c, cudaGetLastError(), "tensor-core receive") ? MLF_OK : MLF_E_CUDA;
}

// the preconditioner's operand layout is stale once its blocks are rebuilt
void tc_drop_precond(Ctx* c) {
    TcState* t = c->tc;
    if (!t) return;
    if (t->M.hi) cudaFree(t->M.hi);
    if (t->M.lo) cudaFree(t->M.lo);
    t->M.hi = t->M.lo = nullptr;
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
