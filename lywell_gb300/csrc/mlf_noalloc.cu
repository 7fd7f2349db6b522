// Allocation-free MLFMA matvec: mlf_matvec_device_noalloc.
//
// Some callers cannot call cudaMalloc while they run the solve: a host that
// records its iteration into a CUDA graph, or one whose device memory is
// owned by another runtime or a fixed pool (a Fortran solver that hands this
// library device pointers and forbids it from allocating).  For them this
// entry point issues exactly the launches of mlf_matvec_device's FP64
// operator (fp64_matvec_launch: aggregation, separable interpolation,
// translation, separable anterpolation, receive + complex(8) near SpMV), but
// keeps the per-level C / B / A multipole fields -- the matvec's scratch --
// in one file-scope device array of fixed size instead of the context's
// buffers.  Its results are therefore bit-identical to mlf_matvec_device's.
//
// Rules of use:
//  * the scratch array holds MLF_NOALLOC_SCRATCH_ELEMS complex values
//    (64 MiB); every GPU that loads the library keeps it until exit.  A
//    context whose fields need more is rejected with MLF_E_ARG;
//  * the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current, and keeps it for the
//    life of the process; make that first call before any stream capture,
//    and make no call on a device after resetting it (cudaDeviceReset ends
//    every context on it anyway);
//  * every call on every context shares the one array and leaves the last
//    call's fields in it; calls that overlap on the GPU (different streams,
//    threads or contexts) race on it.  Nothing needs to start at zero: each
//    stage writes its whole output before the next stage reads it;
//  * the caller's current device is restored before returning.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "mlf_internal.h"

namespace mlf {

constexpr size_t MLF_NOALLOC_SCRATCH_ELEMS = (size_t)64 * 1024 * 1024 / sizeof(double2);
constexpr int MLF_NOALLOC_MAX_DEVICES = 64;

static __device__ __align__(256) double2 g_noalloc_scratch[MLF_NOALLOC_SCRATCH_ELEMS];

namespace {
std::mutex g_lock;
double2* g_scratch_addr[MLF_NOALLOC_MAX_DEVICES] = {nullptr};

// device address of the scratch array on the context's device (current)
double2* scratch_for_device(Ctx* c) {
    std::lock_guard<std::mutex> lk(g_lock);
    if (c->dev < 0 || c->dev >= MLF_NOALLOC_MAX_DEVICES) {
        c->err = "mlf_matvec_device_noalloc: device index " + std::to_string(c->dev) + " is above " +
                 std::to_string(MLF_NOALLOC_MAX_DEVICES - 1);
        return nullptr;
    }
    if (!g_scratch_addr[c->dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (!cuda_ok(c, e, "cudaGetSymbolAddress(scratch)")) return nullptr;
        g_scratch_addr[c->dev] = static_cast<double2*>(p);
    }
    return g_scratch_addr[c->dev];
}

int noalloc_matvec(Ctx* c, const double2* x, double2* y, cudaStream_t s) {
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
    return fp64_matvec_launch(c, x, y, 1, c->N, s, Cf, Bf, Af, nullptr);
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
    int prev = -1;
    if (!cuda_ok(c, cudaGetDevice(&prev), "cudaGetDevice")) return MLF_E_CUDA;
    if (!cuda_ok(c, cudaSetDevice(c->dev), "cudaSetDevice")) return MLF_E_CUDA;
    const int st = noalloc_matvec(c, (const double2*)x_dev, (double2*)y_dev,
                                  stream ? (cudaStream_t)stream : c->stream);
    if (prev != c->dev && !cuda_ok(c, cudaSetDevice(prev), "cudaSetDevice(restore)") && st == MLF_OK)
        return MLF_E_CUDA;
    return st;
}
