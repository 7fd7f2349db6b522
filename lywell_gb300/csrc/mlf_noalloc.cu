// Allocation-free MLFMA matvec: mlf_matvec_device_noalloc.
//
// Some callers cannot call cudaMalloc while they run the solve: a host that
// records its iteration into a CUDA graph, or one whose device memory is
// owned by another runtime or a fixed pool (a Fortran solver that hands this
// library device pointers and forbids it from allocating).  For them this
// entry point runs the same kernels as mlf_matvec_device, but keeps the
// per-level C / B / A multipole fields — the matvec's scratch — in one
// file-scope device array of fixed size instead of the context's buffers.
//
// Rules of use:
//  * the scratch array holds MLF_NOALLOC_SCRATCH_ELEMS complex values
//    (64 MiB); every GPU that loads the library keeps it until exit.  A
//    context whose fields need more is rejected with MLF_E_ARG;
//  * the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current; make that first call
//    before any stream capture;
//  * every call on every context shares the one array and leaves the last
//    call's fields in it; calls that overlap on the GPU (different streams,
//    threads or contexts) race on it.  Nothing needs to start at zero: each
//    stage writes its whole output before the next stage reads it.
#include <cuda_runtime.h>

#include <mutex>

#include "mlf_internal.h"

namespace mlf {

// kernels of mlf_device.cu
__global__ void k_aggregate(int K, int nrhs, int ld, const int* box_ptr, const int* perm, const double2* R,
                            const double2* x, double2* C);
__global__ void k_interp_up(int Kp, int Kc, int nrhs, int nchunk, const int* child_ptr, const int* octant,
                            const double* iw, const int* iidx, const double2* shift, const double2* Cc,
                            double2* Cp);
__global__ void k_translate(int K, int nrhs, int nchunk, const int* far_ptr, const int* far_src,
                            const int* far_tid, const double2* T, const double* wq, const double2* C,
                            double2* B);
__global__ void k_anterp_down(int Kp, int Kc, int nrhs, const int* parent, const int* octant, const int* ant_ptr,
                              const int* ant_row, const double* ant_w, const double2* shift,
                              const double2* Psrc, const double2* Bc, double2* Ac);
__global__ void k_receive_near(int K, int N, int nrhs, int ld, const int* perm, const int* box_of_sorted,
                               const double2* R, const double2* A, const int* ia, const int* ja,
                               const float2* Z, const double2* x, double facy, double2* y);

constexpr size_t MLF_NOALLOC_SCRATCH_ELEMS = (size_t)64 * 1024 * 1024 / sizeof(double2);

static __device__ __align__(256) double2 g_noalloc_scratch[MLF_NOALLOC_SCRATCH_ELEMS];

namespace {
std::mutex g_lock;
double2* g_scratch_addr[64] = {nullptr};

double2* scratch_for_device(Ctx* c) {
    std::lock_guard<std::mutex> lk(g_lock);
    if (c->dev < 0 || c->dev >= 64) return nullptr;
    if (!g_scratch_addr[c->dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (!cuda_ok(c, e, "cudaGetSymbolAddress(scratch)")) return nullptr;
        g_scratch_addr[c->dev] = static_cast<double2*>(p);
    }
    return g_scratch_addr[c->dev];
}
}  // namespace

}  // namespace mlf

using namespace mlf;

extern "C" int mlf_matvec_device_noalloc(mlf_ctx* h, const void* x_dev, void* y_dev, void* stream) {
    if (!h || !x_dev || !y_dev) return MLF_E_ARG;
    Ctx* c = &h->c;
    if (need_tree(c)) return MLF_E_STATE;
    if (c->nlev == 3) {
        c->err = "mlf_matvec_device_noalloc: single-level FMM contexts are not supported";
        return MLF_E_STATE;
    }
    if (!cuda_ok(c, cudaSetDevice(c->dev), "cudaSetDevice")) return MLF_E_CUDA;
    const int nl = c->nlev;
    size_t need = 0;
    for (int n = 3; n <= nl; ++n) need += (size_t)(n >= 4 ? 3 : 2) * c->lv[n].nb * 2 * c->lv[n].K;
    if (need > MLF_NOALLOC_SCRATCH_ELEMS) {
        c->err = "mlf_matvec_device_noalloc: the multipole fields of this octree need " + std::to_string(need) +
                 " complex values, more than the fixed scratch of " +
                 std::to_string(MLF_NOALLOC_SCRATCH_ELEMS) + " (64 MiB); use mlf_matvec_device";
        return MLF_E_ARG;
    }
    double2* base = scratch_for_device(c);
    if (!base) return MLF_E_CUDA;
    double2* Cf[32] = {nullptr};
    double2* Bf[32] = {nullptr};
    double2* Af[32] = {nullptr};
    size_t off = 0;
    for (int n = 3; n <= nl; ++n) {
        const size_t f = (size_t)c->lv[n].nb * 2 * c->lv[n].K;
        Cf[n] = base + off; off += f;
        Bf[n] = base + off; off += f;
        if (n >= 4) { Af[n] = base + off; off += f; }
    }
    cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
    const double2* x = (const double2*)x_dev;
    double2* y = (double2*)y_dev;
    Level& leaf = c->lv[nl];
    k_aggregate<<<leaf.nb, 256, 0, s>>>(leaf.K, 1, c->N, c->dbox_ptr, c->dperm, c->dR, x, Cf[nl]);
    for (int n = nl; n >= 4; --n) {
        Level& Lc = c->lv[n];
        Level& Lp = c->lv[n - 1];
        const int nch = (2 * Lp.K + 255) / 256;
        k_interp_up<<<Lp.nb * nch, 256, 0, s>>>(Lp.K, Lc.K, 1, nch, Lp.dchild_ptr, Lc.doctant, Lp.diw, Lp.diidx,
                                                Lp.dshift, Cf[n], Cf[n - 1]);
    }
    for (int n = 3; n <= nl; ++n) {
        Level& L = c->lv[n];
        const int nch = (2 * L.K + 127) / 128;
        k_translate<<<L.nb * nch, 128, 0, s>>>(L.K, 1, nch, L.dfar_ptr, L.dfar_src, L.dfar_tid, L.dT, L.dwq, Cf[n],
                                               Bf[n]);
    }
    for (int n = 4; n <= nl; ++n) {
        Level& Lc = c->lv[n];
        Level& Lp = c->lv[n - 1];
        const double2* Psrc = (n == 4) ? Bf[n - 1] : Af[n - 1];
        const size_t smem = 2 * (size_t)Lp.K * sizeof(double2);
        k_anterp_down<<<Lc.nb, 256, smem, s>>>(Lp.K, Lc.K, 1, Lc.dparent, Lc.doctant, Lp.dant_ptr, Lp.dant_row,
                                               Lp.dant_w, Lp.dshift, Psrc, Bf[n], Af[n]);
    }
    const double facy = c->ph.w * MU / (4. * PI);
    k_receive_near<<<(c->N * 32 + 255) / 256, 256, 0, s>>>(leaf.K, c->N, 1, c->N, c->dperm, c->dbox_of_sorted,
                                                           c->dR, Af[nl], c->dia, c->dja, c->dZ, x, facy, y);
    return cuda_ok(c, cudaGetLastError(), "mlf_matvec_device_noalloc") ? MLF_OK : MLF_E_CUDA;
}
