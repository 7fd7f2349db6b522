// Block-size and tile autotuner for batched solves.
//
// For each candidate number of right-hand sides per block B, each
// multi-column engine -- the box-block GEMMs (tensor-core mma.sync 3xTF32 or
// FP32 FMA) at each tile width (8, 32 or 64 columns), the warp-per-basis
// engine, and the box blocks with the near field on tcgen05 -- one FP32
// operator application on B random columns is timed with CUDA events (two
// warm-up calls, three timed).
// Engines far outside their range are not timed: the warp engines when leaf
// boxes hold 96 bases or more on average (twice the size below which they
// are the default), the tcgen05 engine below 16 (its tiles pad a box to 16
// rows and its chunks to 32 bases).
// The choice minimises operator time per right-hand side; a smaller block is
// kept when it is within 5 % of the best (it retires columns sooner and holds
// a smaller Krylov basis).  No counterpart in the reference, whose monostatic
// sweep solves one angle at a time (gen_rcs_monostatica, main.f90:967-1089).
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "mlf_internal.h"

namespace mlf {

#define CK(call)                                             \
    do {                                                     \
        if (!cuda_ok(c, (call), #call)) return MLF_E_CUDA;   \
    } while (0)

__global__ void k_fill_pattern(size_t n, double2* __restrict__ x) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    // deterministic, well-spread values in [-1, 1]
    const unsigned h = (unsigned)(i * 2654435761u) ^ (unsigned)(i >> 7);
    x[i] = make_double2(((h & 0xffff) / 32767.5) - 1.0, (((h >> 16) & 0xffff) / 32767.5) - 1.0);
}

int autotune_block(Ctx* c, const int* cand, int ncand, int* best_block, int* best_cols, int* best_engine,
                   float* per_rhs_ms) {
    DevScope ds;
    int bmax = 0;
    for (int q = 0; q < ncand; ++q) bmax = std::max(bmax, cand[q]);
    if (bmax <= 0) return MLF_E_ARG;
    cudaStream_t s = c->stream;
    double2 *x = nullptr, *y = nullptr;
    const size_t n = (size_t)c->N * bmax;
    CK(ds.alloc(&x, n * sizeof(double2)));
    CK(ds.alloc(&y, n * sizeof(double2)));
    k_fill_pattern<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, x);
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    const int saved_cols = c->blk_cols, saved_eng = c->blk_engine, saved_prof = c->profiling;
    c->profiling = 0;
    int st = MLF_OK;
    double best = 1e300;
    *best_block = cand[0];
    *best_cols = 0;
    std::vector<std::pair<double, int>> per(ncand);
    std::vector<int> colsel(ncand, 0), engsel(ncand, 1);
    const long long nbox = std::max<long long>(1, (long long)c->box_ptr.size() - 1);
    const double mean_box = (double)c->N / (double)nbox;
    for (int q = 0; q < ncand && !st; ++q) {
        const int B = cand[q];
        double tq = 1e300;
        const int widths[3] = {8, 32, 64};
        for (int var = 0; var < 9 && !st; ++var) {
            // mma.sync box blocks, FP32 FMA box blocks (three widths each), the warp engine
            // with its per-box and its per-basis receive, then the tcgen05 near field
            const int wv = var % 3, eng = var >= 6 ? var - 4 : 1 - var / 3;
            if (B == 1 && var) break;   // one column uses the CSR kernels
            if ((eng == 2 || eng == 3) && mean_box >= 96.0) continue;
            if (eng == 4 && mean_box < 16.0) continue;
            if (eng < 2 && wv > 0 && widths[wv - 1] >= B) continue;   // a narrower tile already covers the block
            c->blk_cols = eng >= 2 ? 0 : widths[wv];
            c->blk_engine = eng;
            for (int w = 0; w < 2 && !st; ++w) st = device_matvec32(c, x, y, B, c->N, s);
            if (st) break;
            cudaEventRecord(e0, s);
            for (int w = 0; w < 3 && !st; ++w) st = device_matvec32(c, x, y, B, c->N, s);
            cudaEventRecord(e1, s);
            if (st) break;
            if (!cuda_ok(c, cudaEventSynchronize(e1), "autotune")) { st = MLF_E_CUDA; break; }
            if (eng == 4 && (st = tc_check(c))) break;
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            const double t = ms / 3.0 / B;
            if (t < tq) { tq = t; colsel[q] = eng >= 2 ? 0 : widths[wv]; engsel[q] = eng; }
        }
        per[q] = {tq, B};
        if (per_rhs_ms) per_rhs_ms[q] = (float)tq;
        best = std::min(best, tq);
    }
    if (!st) {
        // smallest block within 5 % of the best per-column time
        int pick = -1;
        for (int q = 0; q < ncand; ++q)
            if (per[q].first <= 1.05 * best && (pick < 0 || cand[q] < cand[pick])) pick = q;
        *best_block = cand[pick];
        *best_cols = cand[pick] == 1 ? 0 : colsel[pick];
        c->blk_engine = engsel[pick];
        if (best_engine) *best_engine = engsel[pick];
    } else {
        c->blk_engine = saved_eng;
    }
    c->blk_cols = st ? saved_cols : *best_cols;
    c->profiling = saved_prof;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return st;
}

}  // namespace mlf

using namespace mlf;

extern "C" int mlf_set_block_engine(mlf_ctx* h, int engine, int cols) {
    if (!h || engine < -1 || engine > 4 || (cols != 0 && cols != 8 && cols != 32 && cols != 64)) return MLF_E_ARG;
    h->c.blk_engine = engine;
    h->c.blk_cols = cols;
    return MLF_OK;
}

extern "C" int mlf_autotune_block(mlf_ctx* h, const int* candidates, int ncand, int* best_block, int* best_cols,
                                  int* best_engine, float* per_rhs_ms) {
    if (!h || !candidates || ncand <= 0 || !best_block || !best_cols) return MLF_E_ARG;
    for (int q = 0; q < ncand; ++q)
        if (candidates[q] <= 0 || candidates[q] > 4096) return MLF_E_ARG;
    Ctx* c = &h->c;
    if (!cuda_ok(c, cudaSetDevice(c->dev), "cudaSetDevice")) return MLF_E_CUDA;
    return autotune_block(c, candidates, ncand, best_block, best_cols, best_engine, per_rhs_ms);
}
