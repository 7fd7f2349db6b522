// extern "C" entry points declared in include/lywell_mlfma.h.  Host arrays
// cross the boundary in the reference's Fortran layout (column-major,
// 1-based indices, interleaved complex); this file converts, copies to the
// device and calls the device drivers.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "mlf_internal.h"

using namespace mlf;

namespace {
thread_local std::string g_init_error;

#define CK(call)                                             \
    do {                                                     \
        if (!cuda_ok(c, (call), #call)) return MLF_E_CUDA;   \
    } while (0)

int ensure_io(Ctx* c, size_t n) {
    if (c->io_cap >= n) return MLF_OK;
    if (c->dx_io) cudaFree(c->dx_io);
    if (c->dy_io) cudaFree(c->dy_io);
    c->dx_io = c->dy_io = nullptr;
    CK(cudaMalloc(&c->dx_io, n * sizeof(double2)));
    CK(cudaMalloc(&c->dy_io, n * sizeof(double2)));
    c->io_cap = n;
    return MLF_OK;
}

// host (ld x nrhs) -> device packed (N x nrhs)
int h2d_cols(Ctx* c, double2* dst, const double* src, int nrhs, int ld) {
    if (ld == c->N) {
        CK(cudaMemcpyAsync(dst, src, (size_t)c->N * nrhs * sizeof(double2), cudaMemcpyHostToDevice, c->stream));
    } else {
        CK(cudaMemcpy2DAsync(dst, (size_t)c->N * sizeof(double2), src, (size_t)ld * sizeof(double2),
                             (size_t)c->N * sizeof(double2), nrhs, cudaMemcpyHostToDevice, c->stream));
    }
    return MLF_OK;
}

int d2h_cols(Ctx* c, double* dst, const double2* src, int nrhs, int ld) {
    if (ld == c->N) {
        CK(cudaMemcpyAsync(dst, src, (size_t)c->N * nrhs * sizeof(double2), cudaMemcpyDeviceToHost, c->stream));
    } else {
        CK(cudaMemcpy2DAsync(dst, (size_t)ld * sizeof(double2), src, (size_t)c->N * sizeof(double2),
                             (size_t)c->N * sizeof(double2), nrhs, cudaMemcpyDeviceToHost, c->stream));
    }
    return MLF_OK;
}

bool bind_device(Ctx* c) { return cuda_ok(c, cudaSetDevice(c->dev), "cudaSetDevice"); }
}  // namespace

extern "C" {

int mlf_init(mlf_ctx** out, const double* e_centro, int N, const int* e_t, const int* e_po,
             const double* e_long, const double* t_area, const double* t_baric, const double* t_baric_sub,
             const double* p_coord, const int* t_p, const int* e_p, int P, int T, const double* t_normal,
             double lambda, double ladomax, int flags) {
    (void)t_area; (void)t_p; (void)e_p; (void)t_normal;
    g_init_error.clear();
    if (!out || !e_centro || !e_t || !e_po || !e_long || !t_baric || !t_baric_sub || !p_coord || N <= 0 ||
        P <= 0 || T <= 0 || !(lambda > 0) || !(ladomax > 0)) {
        g_init_error = "invalid argument";
        return MLF_E_ARG;
    }
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        g_init_error = "no CUDA device";
        return MLF_E_NO_DEVICE;
    }
    mlf_ctx* h = new (std::nothrow) mlf_ctx;
    if (!h) return MLF_E_NOMEM;
    Ctx* c = &h->c;
    cudaGetDevice(&c->dev);
    c->N = N; c->P = P; c->T = T;
    c->flags = flags;
    c->ladomax = ladomax;
    c->ph = phys_from_lambda(lambda);
    c->p_coord.assign(p_coord, p_coord + 3 * (size_t)P);
    c->t_baric.assign(t_baric, t_baric + 3 * (size_t)T);
    c->t_baric_sub.assign(t_baric_sub, t_baric_sub + 27 * (size_t)T);
    c->e_long.assign(e_long, e_long + N);
    c->e_centro.assign(e_centro, e_centro + 3 * (size_t)N);
    c->e_t.resize(2 * (size_t)N);
    c->e_po.resize(2 * (size_t)N);
    for (size_t i = 0; i < 2 * (size_t)N; ++i) {
        c->e_t[i] = e_t[i] - 1;
        c->e_po[i] = e_po[i] - 1;
        if (c->e_t[i] < 0 || c->e_t[i] >= T || c->e_po[i] < 0 || c->e_po[i] >= P) {
            g_init_error = "index out of range in e_t / e_po";
            delete h;
            return MLF_E_ARG;
        }
    }
    int st;
    if (flags & MLF_FLAG_DENSE_MOM) {
        c->dense = 1;
        st = dense_setup(c);
    } else {
        st = (flags & MLF_FLAG_FMM) ? build_fmm(c) : build_octree(c);
        if (st == MLF_OK) st = configure_kernels(c);
        if (st == MLF_OK) st = device_setup(c);
    }
    if (st != MLF_OK) {
        g_init_error = c->err;
        device_free(c);
        delete h;
        return st;
    }
    *out = h;
    return MLF_OK;
}

void mlf_free(mlf_ctx* h) {
    if (!h) return;
    cudaSetDevice(h->c.dev);
    device_free(&h->c);
    delete h;
}

const char* mlf_last_error(const mlf_ctx* h) { return h ? h->c.err.c_str() : g_init_error.c_str(); }

int mlf_matvec(mlf_ctx* h, const double* x, double* y, int nrhs, int ld) {
    if (!h || !x || !y || nrhs <= 0 || ld < h->c.N) return MLF_E_ARG;
    Ctx* c = &h->c;
    if (!bind_device(c)) return MLF_E_CUDA;
    const size_t n = (size_t)c->N * nrhs;
    int st;
    if ((st = ensure_io(c, n))) return st;
    if ((st = h2d_cols(c, c->dx_io, x, nrhs, ld))) return st;
    if ((st = device_matvec(c, c->dx_io, c->dy_io, nrhs, c->N, c->stream))) return st;
    if ((st = d2h_cols(c, y, c->dy_io, nrhs, ld))) return st;
    CK(cudaStreamSynchronize(c->stream));
    return MLF_OK;
}

int mlf_matvec_device(mlf_ctx* h, const void* x, void* y, int nrhs, int ld, void* stream) {
    if (!h || !x || !y || nrhs <= 0 || ld < h->c.N) return MLF_E_ARG;
    Ctx* c = &h->c;
    if (!bind_device(c)) return MLF_E_CUDA;
    cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
    return device_matvec(c, (const double2*)x, (double2*)y, nrhs, ld, s);
}

int mlf_near_csr(mlf_ctx* h, long long* nnz, float* a, int* ja, int* ia) {
    if (!h || !nnz) return MLF_E_ARG;
    Ctx* c = &h->c;
    if (need_tree(c)) return MLF_E_STATE;
    *nnz = c->nnz;
    if (!a && !ja && !ia) return MLF_OK;
    if (!bind_device(c)) return MLF_E_CUDA;
    if (a) CK(cudaMemcpy(a, c->dZ, c->nnz * sizeof(float2), cudaMemcpyDeviceToHost));
    if (ja)
        for (long long q = 0; q < c->nnz; ++q) ja[q] = c->ja[q] + 1;
    if (ia)
        for (int i = 0; i <= c->N; ++i) ia[i] = c->ia[i] + 1;
    return MLF_OK;
}

int mlf_ilu0(mlf_ctx* h, int* ierr_row) {
    if (!h || !ierr_row) return MLF_E_ARG;
    Ctx* c = &h->c;
    if (need_tree(c)) return MLF_E_STATE;
    if (!bind_device(c)) return MLF_E_CUDA;
    c->ilu_ok = 0;
    const int ierr = ilu0_factor(c);
    if (ierr < 0) return MLF_E_CUDA;
    *ierr_row = ierr;
    if (ierr != 0) return MLF_OK;
    ilu_levels(c);
    const int st = device_ilu_upload(c);
    if (st) return st;
    c->ilu_ok = 1;
    return MLF_OK;
}

int mlf_ilu0_csr(int n, const float* a, const int* ja, const int* ia, float* alu, int* jlu, int* ju, int* ierr) {
    g_init_error.clear();
    if (n <= 0 || !a || !ja || !ia || !alu || !jlu || !ju || !ierr) {
        g_init_error = "invalid argument";
        return MLF_E_ARG;
    }
    // the CSR must be well formed: ia(1) = 1, ia non-decreasing, columns in
    // 1..n and strictly ascending within each row (ilu0C relies on the L
    // entries preceding the diagonal and checks none of this)
    if (ia[0] != 1) {
        g_init_error = "ia(1) must be 1";
        return MLF_E_ARG;
    }
    for (int i = 0; i < n; ++i) {
        if (ia[i + 1] < ia[i]) {
            g_init_error = "ia decreases at row " + std::to_string(i + 1);
            return MLF_E_ARG;
        }
        for (int q = ia[i] - 1; q < ia[i + 1] - 1; ++q) {
            if (ja[q] < 1 || ja[q] > n) {
                g_init_error = "column index out of range in row " + std::to_string(i + 1);
                return MLF_E_ARG;
            }
            if (q > ia[i] - 1 && ja[q] <= ja[q - 1]) {
                g_init_error = "columns not strictly ascending in row " + std::to_string(i + 1);
                return MLF_E_ARG;
            }
        }
    }
    const long long nnz = (long long)ia[n] - 1;
    std::vector<int> ia0(n + 1), ja0(nnz);
    for (int i = 0; i <= n; ++i) ia0[i] = ia[i] - 1;
    for (long long q = 0; q < nnz; ++q) ja0[q] = ja[q] - 1;
    std::vector<float2> aluv(nnz + 2, make_float2(0.f, 0.f));
    std::vector<int> jluv(nnz + 2, 0), juv(n + 1, 0);
    *ierr = ilu0_msr(n, ia0.data(), ja0.data(), reinterpret_cast<const float2*>(a), aluv.data(), jluv.data(),
                     juv.data());
    // element k of the Fortran arrays alu(nnz+1), jlu(nnz+1), ju(n) is index k here
    std::memcpy(alu, aluv.data() + 1, (size_t)(nnz + 1) * sizeof(float2));
    std::memcpy(jlu, jluv.data() + 1, (size_t)(nnz + 1) * sizeof(int));
    std::memcpy(ju, juv.data() + 1, (size_t)n * sizeof(int));
    return MLF_OK;
}

int mlf_set_near_values(mlf_ctx* h, const float* a) {
    if (!h || !a) return MLF_E_ARG;
    Ctx* c = &h->c;
    if (need_tree(c)) return MLF_E_STATE;
    if (!bind_device(c)) return MLF_E_CUDA;
    return device_set_near(c, reinterpret_cast<const float2*>(a));
}

int mlf_set_stagnation(mlf_ctx* h, int window) {
    if (!h || window < 0) return MLF_E_ARG;
    h->c.stag_window = window;
    return MLF_OK;
}

int mlf_ilut(mlf_ctx* h, double fill_in_prc, double droptol, int* ierr_out) {
    if (!h || !ierr_out || fill_in_prc < 0 || droptol < 0) return MLF_E_ARG;
    Ctx* c = &h->c;
    if (need_tree(c)) return MLF_E_STATE;
    if (!bind_device(c)) return MLF_E_CUDA;
    c->ilu_ok = 0;
    // crear_precond (main.f90:904-906): lfil = ceiling(0.01 * fill_in_prc * N)
    const int lfil = (int)std::ceil(0.01 * fill_in_prc * c->N);
    const int ierr = ilut_factor(c, lfil, droptol);
    if (ierr == -100) return MLF_E_CUDA;
    *ierr_out = ierr;
    if (ierr != 0) return MLF_OK;
    ilu_levels(c);
    const int st = device_ilu_upload(c);
    if (st) return st;
    c->ilu_ok = 1;
    return MLF_OK;
}

int mlf_ilu_size(mlf_ctx* h, long long* len) {
    if (!h || !len) return MLF_E_ARG;
    Ctx* c = &h->c;
    if (!c->ilu_ok) { c->err = "no ILU factors"; return MLF_E_STATE; }
    *len = (long long)c->jlu[c->N + 1] - 1;
    return MLF_OK;
}

int mlf_ilu0_factors(mlf_ctx* h, float* alu, int* jlu, int* ju) {
    if (!h || !alu || !jlu || !ju) return MLF_E_ARG;
    Ctx* c = &h->c;
    if (need_tree(c)) return MLF_E_STATE;
    if (!c->ilu_ok) { c->err = "ILU0 factors not available"; return MLF_E_STATE; }
    // MSR arrays are 1-based: element k of the Fortran array is index k here
    const long long n1 = (long long)c->jlu[c->N + 1] - 1;
    std::memcpy(alu, c->alu.data() + 1, n1 * sizeof(float2));
    std::memcpy(jlu, c->jlu.data() + 1, n1 * sizeof(int));
    std::memcpy(ju, c->ju.data() + 1, (size_t)c->N * sizeof(int));
    return MLF_OK;
}

int mlf_ilu0_solve(mlf_ctx* h, const double* y, double* x, int nrhs) {
    if (!h || !y || !x || nrhs <= 0) return MLF_E_ARG;
    Ctx* c = &h->c;
    if (need_tree(c)) return MLF_E_STATE;
    if (!bind_device(c)) return MLF_E_CUDA;
    const size_t n = (size_t)c->N * nrhs;
    int st;
    if ((st = ensure_io(c, n))) return st;
    if ((st = h2d_cols(c, c->dx_io, y, nrhs, c->N))) return st;
    for (int r = 0; r < nrhs; ++r)
        if ((st = device_ilu_solve(c, c->dx_io + (size_t)r * c->N, c->dy_io + (size_t)r * c->N, c->stream)))
            return st;
    if ((st = d2h_cols(c, x, c->dy_io, nrhs, c->N))) return st;
    CK(cudaStreamSynchronize(c->stream));
    return MLF_OK;
}

int mlf_cgs(mlf_ctx* h, const double* b, const double* x0, double tol, int maxit, int nrhs, double* x,
            int* iters, double* relres, int precond_kind, int* status_out) {
    DevScope ds;
    if (!h || !b || !x || !iters || !relres || !status_out || nrhs <= 0 || maxit <= 0 || !(tol > 0))
        return MLF_E_ARG;
    Ctx* c = &h->c;
    if (precond_kind < 0 || precond_kind > 2) return MLF_E_ARG;
    if (precond_kind == 1 && !c->ilu_ok) { c->err = "ILU0 requested but not factorised"; return MLF_E_STATE; }
    if (precond_kind == 2 && !c->nearinv_ok) {
        c->err = "neighbourhood inverse requested but not built";
        return MLF_E_STATE;
    }
    if (!bind_device(c)) return MLF_E_CUDA;
    const size_t n = (size_t)c->N * nrhs;
    double2 *db = nullptr, *dx = nullptr, *dx0 = nullptr;
    CK(ds.alloc(&db, n * sizeof(double2)));
    CK(ds.alloc(&dx, n * sizeof(double2)));
    int st = h2d_cols(c, db, b, nrhs, c->N);
    if (!st && x0) {
        CK(ds.alloc(&dx0, n * sizeof(double2)));
        st = h2d_cols(c, dx0, x0, nrhs, c->N);
    }
    if (!st) st = device_cgs(c, db, dx0, tol, maxit, nrhs, dx, iters, relres, precond_kind, status_out);
    if (!st) st = d2h_cols(c, x, dx, nrhs, c->N);
    if (!st) CK(cudaStreamSynchronize(c->stream));
    return st;
}

int mlf_solve(mlf_ctx* h, const double* b, const double* x0, double tol, int maxit, int nrhs, int precond_kind,
              int mode, double inner_tol, double* x, int* iters, double* relres, int* status_out, int* outer) {
    DevScope ds;
    if (!h || !b || !x || !iters || !relres || !status_out || nrhs <= 0 || maxit <= 0 || !(tol > 0)) return MLF_E_ARG;
    if (mode != 0 && mode != 1) return MLF_E_ARG;
    if (mode == 0) {
        if (outer) *outer = 0;
        return mlf_cgs(h, b, x0, tol, maxit, nrhs, x, iters, relres, precond_kind, status_out);
    }
    Ctx* c = &h->c;
    if (precond_kind < 0 || precond_kind > 2) return MLF_E_ARG;
    if ((precond_kind == 1 && !c->ilu_ok) || (precond_kind == 2 && !c->nearinv_ok)) {
        c->err = "requested preconditioner not built";
        return MLF_E_STATE;
    }
    if (!bind_device(c)) return MLF_E_CUDA;
    const size_t n = (size_t)c->N * nrhs;
    double2 *db = nullptr, *dx = nullptr, *dx0 = nullptr;
    CK(ds.alloc(&db, n * sizeof(double2)));
    CK(ds.alloc(&dx, n * sizeof(double2)));
    int st = h2d_cols(c, db, b, nrhs, c->N);
    if (!st && x0) {
        CK(ds.alloc(&dx0, n * sizeof(double2)));
        st = h2d_cols(c, dx0, x0, nrhs, c->N);
    }
    int outer_k = 0;
    if (!st)
        st = device_solve_mixed(c, db, dx0, tol, maxit, nrhs, dx, iters, relres, precond_kind, status_out,
                                inner_tol > 0 ? inner_tol : 0.9 * tol, &outer_k);
    if (outer) *outer = outer_k;
    if (!st) st = d2h_cols(c, x, dx, nrhs, c->N);
    if (!st) CK(cudaStreamSynchronize(c->stream));
    return st;
}

int mlf_matvec32(mlf_ctx* h, const double* x, double* y, int nrhs, int ld) {
    if (!h || !x || !y || nrhs <= 0 || ld < h->c.N) return MLF_E_ARG;
    Ctx* c = &h->c;
    if (!bind_device(c)) return MLF_E_CUDA;
    const size_t n = (size_t)c->N * nrhs;
    int st;
    if ((st = ensure_io(c, n))) return st;
    if ((st = h2d_cols(c, c->dx_io, x, nrhs, ld))) return st;
    if ((st = device_matvec32(c, c->dx_io, c->dy_io, nrhs, c->N, c->stream))) return st;
    if ((st = d2h_cols(c, y, c->dy_io, nrhs, ld))) return st;
    CK(cudaStreamSynchronize(c->stream));
    return blk_engine_of(c) == 4 ? tc_check(c) : MLF_OK;
}

int mlf_cgs_history(mlf_ctx* h, int col, double* hist, int cap, int* n) {
    if (!h || !n) return MLF_E_ARG;
    Ctx* c = &h->c;
    const int nr = std::max(c->cgs_hist_nrhs, 1);
    if (col < 0 || col >= nr) return MLF_E_ARG;
    const int total = (int)(c->cgs_hist.size() / nr);
    *n = total;
    if (hist)
        for (int i = 0; i < std::min(cap, total); ++i) hist[i] = c->cgs_hist[(size_t)i * nr + col];
    return MLF_OK;
}

int mlf_precond_apply(mlf_ctx* h, int precond_kind, const double* y, double* x, int nrhs) {
    if (!h || !y || !x || nrhs <= 0 || precond_kind < 1 || precond_kind > 2) return MLF_E_ARG;
    Ctx* c = &h->c;
    if (!bind_device(c)) return MLF_E_CUDA;
    const size_t n = (size_t)c->N * nrhs;
    int st;
    if ((st = ensure_io(c, n))) return st;
    if ((st = h2d_cols(c, c->dx_io, y, nrhs, c->N))) return st;
    if (precond_kind == 2) {
        if ((st = device_nearinv_apply(c, c->dx_io, c->dy_io, nrhs, c->stream))) return st;
    } else {
        for (int r = 0; r < nrhs; ++r)
            if ((st = device_ilu_solve(c, c->dx_io + (size_t)r * c->N, c->dy_io + (size_t)r * c->N, c->stream)))
                return st;
    }
    if ((st = d2h_cols(c, x, c->dy_io, nrhs, c->N))) return st;
    CK(cudaStreamSynchronize(c->stream));
    return MLF_OK;
}

namespace {
__global__ void k_cast_df(size_t n, const double2* __restrict__ a, float2* __restrict__ b) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) b[i] = make_float2((float)a[i].x, (float)a[i].y);
}
__global__ void k_cast_fd(size_t n, const float2* __restrict__ a, double2* __restrict__ b) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) b[i] = make_double2(a[i].x, a[i].y);
}
}  // namespace

int mlf_precond_apply32(mlf_ctx* h, const double* y, double* x, int nrhs) {
    DevScope ds;
    if (!h || !y || !x || nrhs <= 0) return MLF_E_ARG;
    Ctx* c = &h->c;
    if (!bind_device(c)) return MLF_E_CUDA;
    const size_t n = (size_t)c->N * nrhs;
    int st;
    if ((st = ensure_io(c, n))) return st;
    if ((st = h2d_cols(c, c->dx_io, y, nrhs, c->N))) return st;
    float2 *a = nullptr, *b = nullptr;
    CK(ds.alloc(&a, n * sizeof(float2)));
    CK(ds.alloc(&b, n * sizeof(float2)));
    const unsigned g = (unsigned)((n + 255) / 256);
    k_cast_df<<<g, 256, 0, c->stream>>>(n, c->dx_io, a);
    st = device_nearinv_apply32(c, a, b, nrhs, c->stream);
    if (!st) {
        k_cast_fd<<<g, 256, 0, c->stream>>>(n, b, c->dy_io);
        st = d2h_cols(c, x, c->dy_io, nrhs, c->N);
    }
    if (!st && !cuda_ok(c, cudaStreamSynchronize(c->stream), "precond32")) st = MLF_E_CUDA;
    if (!st && blk_engine_of(c) == 4) st = tc_check(c);
    return st;
}

int mlf_excitation(mlf_ctx* h, const double* dirs, const double* pols, double ctte_re, double ctte_im, int nrhs,
                   double* b) {
    if (!h || !dirs || !pols || !b || nrhs <= 0) return MLF_E_ARG;
    Ctx* c = &h->c;
    if (!bind_device(c)) return MLF_E_CUDA;
    const size_t n = (size_t)c->N * nrhs;
    int st;
    if ((st = ensure_io(c, n))) return st;
    if ((st = device_excitation(c, dirs, (const double2*)pols, make_double2(ctte_re, ctte_im), nrhs, c->dy_io)))
        return st;
    if ((st = d2h_cols(c, b, c->dy_io, nrhs, c->N))) return st;
    CK(cudaStreamSynchronize(c->stream));
    return MLF_OK;
}

int mlf_rcs(mlf_ctx* h, const double* I, const double* pol, double ctte_re, double ctte_im, const double* theta,
            const double* phi, int nang, double* sigma) {
    if (!h || !I || !pol || !theta || !phi || !sigma || nang <= 0) return MLF_E_ARG;
    Ctx* c = &h->c;
    if (!bind_device(c)) return MLF_E_CUDA;
    int st;
    if ((st = ensure_io(c, c->N))) return st;
    if ((st = h2d_cols(c, c->dx_io, I, 1, c->N))) return st;
    return device_rcs(c, c->dx_io, (const double2*)pol, make_double2(ctte_re, ctte_im), theta, phi, nang, sigma);
}

int mlf_info(mlf_ctx* h, int* out, long long* nnz_near) {
    if (!h || !out) return MLF_E_ARG;
    Ctx* c = &h->c;
    out[0] = c->nlev;
    out[1] = c->N; out[2] = 0; out[3] = 0; out[4] = 0;
    for (int l = 1; l <= c->nlev && l < 32; ++l) {
        out[5 * l] = c->lv[l].nb;
        out[5 * l + 1] = c->lv[l].L;
        out[5 * l + 2] = c->lv[l].K;
        out[5 * l + 3] = c->lv[l].ntrans;
        out[5 * l + 4] = l >= 3 ? (int)c->lv[l].far_src.size() : 0;
    }
    if (nnz_near) *nnz_near = c->nnz;
    return MLF_OK;
}

int mlf_set_profiling(mlf_ctx* h, int on) {
    if (!h) return MLF_E_ARG;
    h->c.profiling = on ? 1 : 0;
    return MLF_OK;
}

int mlf_stage_times(mlf_ctx* h, float* out5) {
    if (!h || !out5) return MLF_E_ARG;
    std::memcpy(out5, h->c.stage_ms, 5 * sizeof(float));
    return MLF_OK;
}

int mlf_debug_field(mlf_ctx* h, int level, int which, double* out) {
    if (!h || !out) return MLF_E_ARG;
    Ctx* c = &h->c;
    if (need_tree(c)) return MLF_E_STATE;
    if (level < 3 || level > c->nlev || which < 0 || which > 2) return MLF_E_ARG;
    if (!bind_device(c)) return MLF_E_CUDA;
    Level& L = c->lv[level];
    const double2* src = which == 0 ? L.dC : which == 1 ? L.dB : L.dA;
    if (level == 3 && which == 2) src = L.dB;  // level 3 has no A (the reference never fills it)
    const size_t K2 = 2 * (size_t)L.K;
    // column 0 of a field that may hold several right-hand sides
    CK(cudaMemcpy2D(out, K2 * sizeof(double2), src, K2 * c->last_nrhs * sizeof(double2), K2 * sizeof(double2), L.nb,
                    cudaMemcpyDeviceToHost));
    return MLF_OK;
}

}  // extern "C"
