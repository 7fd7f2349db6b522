// Solver-side kernels: ILU(0) triangular sweeps (level scheduled), the CGS
// iteration with device-resident scalars, the plane-wave excitation and the
// RCS far-field sum.
//
//   lusol0C       modIterativo.f90:504-560   -> k_sweep_fwd / k_sweep_bwd, one
//                 warp per row, rows of one dependency level per launch; the
//                 launches of one application are captured in a CUDA graph.
//   CGSold        modIterativo.f90:331-493   -> device_cgs: per-column scalars
//                 (rho, alpha, beta) live on the device; dot products are
//                 block partial sums reduced in a fixed order (run-to-run
//                 deterministic); columns that converge stop updating.
//   generar_onda  main.f90:1488-1525         -> k_excitation
//   sigmaRCS      modRCS.f90:60-153          -> k_rcs, one block per angle.
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

__device__ __forceinline__ void cmac(double2& acc, double2 a, double2 b) {
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(-a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(a.y, b.x, acc.y);
}
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
    const double d = b.x * b.x + b.y * b.y;
    return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}

// ---------------------------------------------------------------------------
// ILU(0) sweeps on the reference's MSR arrays (1-based content, vectors 0-based)
// ---------------------------------------------------------------------------

__global__ void k_sweep_fwd(const int* __restrict__ rows, int nrows, const int* __restrict__ jlu,
                            const int* __restrict__ ju, const float2* __restrict__ alu,
                            const double2* __restrict__ y, double2* __restrict__ x) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= nrows) return;
    const int i = rows[w];
    double sr = 0, si = 0;
    for (int k = jlu[i] + lane; k < ju[i]; k += 32) {
        const float2 a = alu[k];
        const double2 v = x[jlu[k] - 1];
        sr = fma((double)a.x, v.x, sr); sr = fma(-(double)a.y, v.y, sr);
        si = fma((double)a.x, v.y, si); si = fma((double)a.y, v.x, si);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sr += __shfl_xor_sync(0xffffffff, sr, o);
        si += __shfl_xor_sync(0xffffffff, si, o);
    }
    if (lane == 0) {
        const double2 yi = y[i - 1];
        x[i - 1] = make_double2(yi.x - sr, yi.y - si);
    }
}

__global__ void k_sweep_bwd(const int* __restrict__ rows, int nrows, const int* __restrict__ jlu,
                            const int* __restrict__ ju, const float2* __restrict__ alu,
                            double2* __restrict__ x) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= nrows) return;
    const int i = rows[w];
    double sr = 0, si = 0;
    for (int k = ju[i] + lane; k < jlu[i + 1]; k += 32) {
        const float2 a = alu[k];
        const double2 v = x[jlu[k] - 1];
        sr = fma((double)a.x, v.x, sr); sr = fma(-(double)a.y, v.y, sr);
        si = fma((double)a.x, v.y, si); si = fma((double)a.y, v.x, si);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sr += __shfl_xor_sync(0xffffffff, sr, o);
        si += __shfl_xor_sync(0xffffffff, si, o);
    }
    if (lane == 0) {
        const double2 xi = x[i - 1];
        const double2 t = make_double2(xi.x - sr, xi.y - si);
        const float2 d = alu[i];
        x[i - 1] = make_double2((double)d.x * t.x - (double)d.y * t.y, (double)d.x * t.y + (double)d.y * t.x);
    }
}

int device_ilu_upload(Ctx* c) {
    auto F = [](void* p) { if (p) cudaFree(p); };
    F(c->dalu); F(c->djlu); F(c->dju); F(c->dlvl_rows_f); F(c->dlvl_rows_b);
    CK(cudaMalloc(&c->dalu, c->alu.size() * sizeof(float2)));
    CK(cudaMemcpy(c->dalu, c->alu.data(), c->alu.size() * sizeof(float2), cudaMemcpyHostToDevice));
    CK(cudaMalloc(&c->djlu, c->jlu.size() * sizeof(int)));
    CK(cudaMemcpy(c->djlu, c->jlu.data(), c->jlu.size() * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMalloc(&c->dju, c->ju.size() * sizeof(int)));
    CK(cudaMemcpy(c->dju, c->ju.data(), c->ju.size() * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMalloc(&c->dlvl_rows_f, c->lvl_rows_f.size() * sizeof(int)));
    CK(cudaMemcpy(c->dlvl_rows_f, c->lvl_rows_f.data(), c->lvl_rows_f.size() * sizeof(int),
                  cudaMemcpyHostToDevice));
    CK(cudaMalloc(&c->dlvl_rows_b, c->lvl_rows_b.size() * sizeof(int)));
    CK(cudaMemcpy(c->dlvl_rows_b, c->lvl_rows_b.data(), c->lvl_rows_b.size() * sizeof(int),
                  cudaMemcpyHostToDevice));
    return MLF_OK;
}

// x = (LU)^-1 y for one column; y and x must not alias.
int device_ilu_solve(Ctx* c, const double2* y, double2* x, cudaStream_t s) {
    if (!c->ilu_ok) {
        c->err = "ILU0 factors not available (mlf_ilu0 has not succeeded)";
        return MLF_E_STATE;
    }
    const int nlf = (int)c->lvl_ptr_f.size() - 1, nlb = (int)c->lvl_ptr_b.size() - 1;
    for (int l = 0; l < nlf; ++l) {
        const int r0 = c->lvl_ptr_f[l], nr = c->lvl_ptr_f[l + 1] - r0;
        k_sweep_fwd<<<(nr * 32 + 255) / 256, 256, 0, s>>>(c->dlvl_rows_f + r0, nr, c->djlu, c->dju, c->dalu,
                                                          y, x);
    }
    for (int l = 0; l < nlb; ++l) {
        const int r0 = c->lvl_ptr_b[l], nr = c->lvl_ptr_b[l + 1] - r0;
        k_sweep_bwd<<<(nr * 32 + 255) / 256, 256, 0, s>>>(c->dlvl_rows_b + r0, nr, c->djlu, c->dju, c->dalu,
                                                          x);
    }
    return cuda_ok(c, cudaGetLastError(), "ilu sweeps") ? MLF_OK : MLF_E_CUDA;
}

// ---------------------------------------------------------------------------
// CGS
// ---------------------------------------------------------------------------

constexpr int RED_BLOCKS = 256;
constexpr int RED_THREADS = 256;

// per-column scalar block (doubles)
enum {
    S_RHO1 = 0, S_RHO2 = 2, S_ALPHA = 4, S_BETA = 6, S_SV = 8, S_RR = 10, S_BB = 11, S_NSCAL = 12
};
// per-column int flags
enum { F_DONE = 0, F_STATUS = 1, F_ITERS = 2, F_NFLAG = 3 };

// partial sums of sum a*b (unconjugated, mode 0) or sum |a|^2 (mode 1),
// partials[(col*RED_BLOCKS + block)*2]
__global__ void k_dot_partial(int N, const double2* __restrict__ a, const double2* __restrict__ b, int mode,
                              const int* __restrict__ flags, double* __restrict__ partials) {
    const int col = blockIdx.y;
    __shared__ double sr[RED_THREADS], si[RED_THREADS];
    double r = 0, im = 0;
    if (!flags || !flags[col * F_NFLAG + F_DONE]) {
        const double2* ac = a + (size_t)col * N;
        const double2* bc = b + (size_t)col * N;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
            const double2 u = ac[i];
            if (mode == 0) {
                const double2 v = bc[i];
                r = fma(u.x, v.x, r); r = fma(-u.y, v.y, r);
                im = fma(u.x, v.y, im); im = fma(u.y, v.x, im);
            } else {
                r = fma(u.x, u.x, r); r = fma(u.y, u.y, r);
            }
        }
    }
    sr[threadIdx.x] = r;
    si[threadIdx.x] = im;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) { sr[threadIdx.x] += sr[threadIdx.x + s]; si[threadIdx.x] += si[threadIdx.x + s]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partials[((size_t)col * gridDim.x + blockIdx.x) * 2] = sr[0];
        partials[((size_t)col * gridDim.x + blockIdx.x) * 2 + 1] = si[0];
    }
}

__device__ double2 reduce_partials(const double* partials, int col, int nblk) {
    __shared__ double sr[RED_THREADS], si[RED_THREADS];
    double r = 0, im = 0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) {
        r += partials[((size_t)col * nblk + b) * 2];
        im += partials[((size_t)col * nblk + b) * 2 + 1];
    }
    sr[threadIdx.x] = r;
    si[threadIdx.x] = im;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) { sr[threadIdx.x] += sr[threadIdx.x + s]; si[threadIdx.x] += si[threadIdx.x + s]; }
        __syncthreads();
    }
    return make_double2(sr[0], si[0]);
}

__device__ __forceinline__ bool finite2(double2 v) { return isfinite(v.x) && isfinite(v.y); }

// what: 0 = store ||b||^2; 1 = rho1 (start of iteration); 2 = alpha; 3 = residual check
__global__ void k_finalize(int what, int nblk, const double* __restrict__ partials, double* __restrict__ scal,
                           int* __restrict__ flags, double tol2) {
    const int col = blockIdx.x;
    int* fl = flags + col * F_NFLAG;
    if (what != 0 && fl[F_DONE]) return;
    const double2 s = reduce_partials(partials, col, nblk);
    if (threadIdx.x != 0) return;
    double* sc = scal + col * S_NSCAL;
    if (what == 0) {
        sc[S_BB] = s.x;
        return;
    }
    if (what == 1) {
        fl[F_ITERS] += 1;
        if (!finite2(s)) { fl[F_STATUS] = MLF_CGS_NOT_FINITE; fl[F_DONE] = 1; return; }
        if (s.x == 0.0 && s.y == 0.0) { fl[F_STATUS] = MLF_CGS_BREAKDOWN; fl[F_DONE] = 1; return; }
        sc[S_RHO1] = s.x; sc[S_RHO1 + 1] = s.y;
        if (fl[F_ITERS] > 1) {
            const double2 b = cdiv(s, make_double2(sc[S_RHO2], sc[S_RHO2 + 1]));
            sc[S_BETA] = b.x; sc[S_BETA + 1] = b.y;
        }
        return;
    }
    if (what == 2) {
        const double2 a = cdiv(make_double2(sc[S_RHO1], sc[S_RHO1 + 1]), s);
        if (!finite2(a)) { fl[F_STATUS] = MLF_CGS_NOT_FINITE; fl[F_DONE] = 1; return; }
        sc[S_ALPHA] = a.x; sc[S_ALPHA + 1] = a.y;
        return;
    }
    // residual check, ||r|| < tol ||b||  <=>  rr < tol^2 bb
    sc[S_RR] = s.x;
    if (!isfinite(s.x)) { fl[F_STATUS] = MLF_CGS_NOT_FINITE; fl[F_DONE] = 1; return; }
    if (s.x < tol2 * sc[S_BB]) { fl[F_STATUS] = MLF_CGS_CONVERGED; fl[F_DONE] = 1; return; }
    sc[S_RHO2] = sc[S_RHO1]; sc[S_RHO2 + 1] = sc[S_RHO1 + 1];
}

// u = r + beta q ; p = u + beta (q + beta p)   (first iteration: u = r, p = u)
__global__ void k_upd_up(int N, const double2* __restrict__ r, const double2* __restrict__ q,
                         double2* __restrict__ u, double2* __restrict__ p, const double* __restrict__ scal,
                         const int* __restrict__ flags) {
    const int col = blockIdx.y;
    const int* fl = flags + col * F_NFLAG;
    if (fl[F_DONE]) return;
    const size_t o = (size_t)col * N;
    const int first = fl[F_ITERS] == 1;
    const double2 be = make_double2(scal[col * S_NSCAL + S_BETA], scal[col * S_NSCAL + S_BETA + 1]);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const double2 ri = r[o + i];
        if (first) {
            u[o + i] = ri;
            p[o + i] = ri;
        } else {
            const double2 qi = q[o + i];
            const double2 bq = cmul(be, qi);
            const double2 ui = make_double2(ri.x + bq.x, ri.y + bq.y);
            const double2 bp = cmul(be, p[o + i]);
            const double2 t = cmul(be, make_double2(qi.x + bp.x, qi.y + bp.y));
            u[o + i] = ui;
            p[o + i] = make_double2(ui.x + t.x, ui.y + t.y);
        }
    }
}

// q = u - alpha V ; t = u + q
__global__ void k_upd_q(int N, const double2* __restrict__ u, const double2* __restrict__ V,
                        double2* __restrict__ q, double2* __restrict__ t, const double* __restrict__ scal,
                        const int* __restrict__ flags) {
    const int col = blockIdx.y;
    if (flags[col * F_NFLAG + F_DONE]) return;
    const size_t o = (size_t)col * N;
    const double2 al = make_double2(scal[col * S_NSCAL + S_ALPHA], scal[col * S_NSCAL + S_ALPHA + 1]);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const double2 ui = u[o + i];
        const double2 av = cmul(al, V[o + i]);
        const double2 qi = make_double2(ui.x - av.x, ui.y - av.y);
        q[o + i] = qi;
        t[o + i] = make_double2(ui.x + qi.x, ui.y + qi.y);
    }
}

// x += alpha U
__global__ void k_upd_x(int N, const double2* __restrict__ U, double2* __restrict__ x,
                        const double* __restrict__ scal, const int* __restrict__ flags) {
    const int col = blockIdx.y;
    if (flags[col * F_NFLAG + F_DONE]) return;
    const size_t o = (size_t)col * N;
    const double2 al = make_double2(scal[col * S_NSCAL + S_ALPHA], scal[col * S_NSCAL + S_ALPHA + 1]);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const double2 a = cmul(al, U[o + i]);
        x[o + i].x += a.x;
        x[o + i].y += a.y;
    }
}

// r -= alpha Q
__global__ void k_upd_r(int N, const double2* __restrict__ Q, double2* __restrict__ r,
                        const double* __restrict__ scal, const int* __restrict__ flags) {
    const int col = blockIdx.y;
    if (flags[col * F_NFLAG + F_DONE]) return;
    const size_t o = (size_t)col * N;
    const double2 al = make_double2(scal[col * S_NSCAL + S_ALPHA], scal[col * S_NSCAL + S_ALPHA + 1]);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const double2 a = cmul(al, Q[o + i]);
        r[o + i].x -= a.x;
        r[o + i].y -= a.y;
    }
}

// r = b - Ax ; Rt = r
__global__ void k_init_r(int N, const double2* __restrict__ b, const double2* __restrict__ Ax,
                         double2* __restrict__ r, double2* __restrict__ Rt) {
    const size_t o = (size_t)blockIdx.y * N;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const double2 v = make_double2(b[o + i].x - Ax[o + i].x, b[o + i].y - Ax[o + i].y);
        r[o + i] = v;
        Rt[o + i] = v;
    }
}

int ensure_work(Ctx* c, size_t n) {
    if (c->work_cap >= n) return MLF_OK;
    if (c->dwork) cudaFree(c->dwork);
    c->dwork = nullptr;
    CK(cudaMalloc(&c->dwork, n * sizeof(double2)));
    c->work_cap = n;
    return MLF_OK;
}

static int precond_apply(Ctx* c, int precond, int nrhs, const double2* y, double2* x, cudaStream_t s) {
    if (precond == 0) {
        CK(cudaMemcpyAsync(x, y, (size_t)nrhs * c->N * sizeof(double2), cudaMemcpyDeviceToDevice, s));
        return MLF_OK;
    }
    if (precond == 2) return device_nearinv_apply(c, y, x, nrhs, s);
    for (int r = 0; r < nrhs; ++r) {
        const int st = device_ilu_solve(c, y + (size_t)r * c->N, x + (size_t)r * c->N, s);
        if (st) return st;
    }
    return MLF_OK;
}

// b, x0, x: device arrays N x nrhs (ld = N).  x0 may equal nullptr.
int device_cgs(Ctx* c, const double2* b, const double2* x0, double tol, int maxit, int nrhs, double2* x,
               int* iters, double* relres, int precond, int* status) {
    const int N = c->N;
    const size_t V = (size_t)N * nrhs;
    int st;
    if ((st = ensure_work(c, 10 * V))) return st;
    double2* r = c->dwork;
    double2* Rt = r + V;
    double2* u = Rt + V;
    double2* p = u + V;
    double2* Ph = p + V;
    double2* Vv = Ph + V;
    double2* q = Vv + V;
    double2* t = q + V;
    double2* Uh = t + V;
    double2* Qv = Uh + V;
    const size_t nscal = (size_t)nrhs * S_NSCAL + (size_t)nrhs * RED_BLOCKS * 2;
    if (c->scal_cap < nscal) {
        if (c->dscal) cudaFree(c->dscal);
        if (c->dflags) cudaFree(c->dflags);
        CK(cudaMalloc(&c->dscal, nscal * sizeof(double)));
        CK(cudaMalloc(&c->dflags, (size_t)nrhs * F_NFLAG * sizeof(int)));
        c->scal_cap = nscal;
    }
    double* scal = c->dscal;
    double* partials = scal + (size_t)nrhs * S_NSCAL;
    int* flags = c->dflags;
    cudaStream_t s = c->stream;
    CK(cudaMemsetAsync(scal, 0, (size_t)nrhs * S_NSCAL * sizeof(double), s));
    CK(cudaMemsetAsync(flags, 0, (size_t)nrhs * F_NFLAG * sizeof(int), s));
    const dim3 vg(std::min((N + 255) / 256, 1024), nrhs);
    const dim3 rg(RED_BLOCKS, nrhs);
    // r = b - A x0 (the reference applies the operator to the guess, zero or not)
    if (x0) CK(cudaMemcpyAsync(x, x0, V * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    else CK(cudaMemsetAsync(x, 0, V * sizeof(double2), s));
    if ((st = device_matvec(c, x, Qv, nrhs, N, s))) return st;
    k_init_r<<<vg, 256, 0, s>>>(N, b, Qv, r, Rt);
    k_dot_partial<<<rg, RED_THREADS, 0, s>>>(N, b, b, 1, nullptr, partials);
    k_finalize<<<nrhs, RED_THREADS, 0, s>>>(0, RED_BLOCKS, partials, scal, flags, 0.0);
    const double tol2 = tol * tol;
    std::vector<int> hflags((size_t)nrhs * F_NFLAG);
    std::vector<double> hscal((size_t)nrhs * S_NSCAL);
    c->cgs_hist.clear();
    c->cgs_hist_nrhs = nrhs;
    // stagnation: the best residual of each column and the iteration that set it
    std::vector<double> best(nrhs, HUGE_VAL);
    std::vector<int> best_it(nrhs, 0);
    int it = 0;
    for (; it < maxit; ++it) {
        k_dot_partial<<<rg, RED_THREADS, 0, s>>>(N, r, Rt, 0, flags, partials);
        k_finalize<<<nrhs, RED_THREADS, 0, s>>>(1, RED_BLOCKS, partials, scal, flags, tol2);
        k_upd_up<<<vg, 256, 0, s>>>(N, r, q, u, p, scal, flags);
        if ((st = precond_apply(c, precond, nrhs, p, Ph, s))) return st;
        if ((st = device_matvec(c, Ph, Vv, nrhs, N, s))) return st;
        k_dot_partial<<<rg, RED_THREADS, 0, s>>>(N, Rt, Vv, 0, flags, partials);
        k_finalize<<<nrhs, RED_THREADS, 0, s>>>(2, RED_BLOCKS, partials, scal, flags, tol2);
        k_upd_q<<<vg, 256, 0, s>>>(N, u, Vv, q, t, scal, flags);
        if ((st = precond_apply(c, precond, nrhs, t, Uh, s))) return st;
        k_upd_x<<<vg, 256, 0, s>>>(N, Uh, x, scal, flags);
        if ((st = device_matvec(c, Uh, Qv, nrhs, N, s))) return st;
        k_upd_r<<<vg, 256, 0, s>>>(N, Qv, r, scal, flags);
        k_dot_partial<<<rg, RED_THREADS, 0, s>>>(N, r, r, 1, flags, partials);
        k_finalize<<<nrhs, RED_THREADS, 0, s>>>(3, RED_BLOCKS, partials, scal, flags, tol2);
        CK(cudaMemcpyAsync(hflags.data(), flags, hflags.size() * sizeof(int), cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(hscal.data(), scal, hscal.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        bool stalled = false;
        for (int col = 0; col < nrhs; ++col) {
            const double bb = hscal[col * S_NSCAL + S_BB];
            const double rel = bb > 0 ? std::sqrt(hscal[col * S_NSCAL + S_RR] / bb) : 0.0;
            c->cgs_hist.push_back(rel);
            int* fl = &hflags[col * F_NFLAG];
            if (c->stag_window <= 0 || fl[F_DONE]) continue;
            if (rel < best[col]) {
                best[col] = rel;
                best_it[col] = fl[F_ITERS];
            } else if (fl[F_ITERS] - best_it[col] >= c->stag_window) {
                fl[F_DONE] = 1;
                fl[F_STATUS] = MLF_CGS_STAGNATED;
                stalled = true;
            }
        }
        // retire the stagnated columns on the device (the update kernels skip done columns)
        if (stalled)
            CK(cudaMemcpyAsync(flags, hflags.data(), hflags.size() * sizeof(int), cudaMemcpyHostToDevice, s));
        bool all = true;
        for (int col = 0; col < nrhs; ++col) all = all && hflags[col * F_NFLAG + F_DONE];
        if (all) break;
    }
    CK(cudaMemcpyAsync(hflags.data(), flags, hflags.size() * sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(hscal.data(), scal, hscal.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    for (int col = 0; col < nrhs; ++col) {
        const int* fl = &hflags[col * F_NFLAG];
        iters[col] = fl[F_ITERS];
        status[col] = fl[F_DONE] ? fl[F_STATUS] : MLF_CGS_MAXIT;
        const double bb = hscal[col * S_NSCAL + S_BB];
        relres[col] = bb > 0 ? std::sqrt(hscal[col * S_NSCAL + S_RR] / bb) : 0.0;
    }
    return MLF_OK;
}

// ---------------------------------------------------------------------------
// excitation and RCS
// ---------------------------------------------------------------------------

__global__ void k_excitation(int N, int nrhs, const double* __restrict__ dirs, const double2* __restrict__ pols,
                             double2 ctte, const double* __restrict__ p_coord, const double* __restrict__ t_baric,
                             const int* __restrict__ e_t, const int* __restrict__ e_po,
                             const double* __restrict__ e_long, double w_smue, double2* __restrict__ b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = blockIdx.y;
    if (i >= N) return;
    const double* d = dirs + 3 * r;
    const double nd = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    const double u0 = d[0] / nd, u1 = d[1] / nd, u2 = d[2] / nd;
    const double2* pol = pols + 3 * r;
    double2 acc = make_double2(0, 0);
    for (int s = 0; s < 2; ++s) {
        const double* bc = t_baric + 3 * e_t[2 * i + s];
        const double* vo = p_coord + 3 * e_po[2 * i + s];
        const double a = w_smue * (u0 * bc[0] + u1 * bc[1] + u2 * bc[2]);
        double sn, cs;
        sincos(a, &sn, &cs);
        const double2 e = make_double2(cs, -sn);
        for (int k = 0; k < 3; ++k) {
            const double2 oE = cmul(cmul(pol[k], ctte), e);
            const double arm = s == 0 ? bc[k] - vo[k] : vo[k] - bc[k];
            acc.x += oE.x * arm;
            acc.y += oE.y * arm;
        }
    }
    const double l = e_long[i];
    b[(size_t)r * N + i] = make_double2(acc.x * 0.5 * l, acc.y * 0.5 * l);
}

// One CTA per angle a; the currents of angle a are I + a istride (istride 0:
// one current vector for every angle) and its polarisation norm den[a].
__global__ void k_rcs(int N, const double* __restrict__ t_baric, const int* __restrict__ e_t,
                      const double* __restrict__ e_long, const double2* __restrict__ Iall, size_t istride,
                      const double* __restrict__ th, const double* __restrict__ ph, double rx, double ry, double rz,
                      double rzl, double w_smue, double facE, const double* __restrict__ den,
                      double* __restrict__ sigma) {
    const int a = blockIdx.x;
    const double2* __restrict__ I = Iall + (size_t)a * istride;
    double st, ct, sp, cp;
    sincos(th[a], &st, &ct);
    sincos(ph[a], &sp, &cp);
    const double ro[3] = {rx + (rzl * st * cp), ry + (rzl * st * sp), rz + (rzl * ct)};
    double2 E[3] = {{0, 0}, {0, 0}, {0, 0}};
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const double* cpv = t_baric + 3 * e_t[2 * i];
        const double* cmv = t_baric + 3 * e_t[2 * i + 1];
        const double2 Ii = I[i];
        const double l = e_long[i];
        double rm[3], rr[3];
        double2 m[3];
        for (int d = 0; d < 3; ++d) {
            rm[d] = 0.5 * (cpv[d] + cmv[d]);
            const double dd = (cmv[d] - cpv[d]);
            m[d] = make_double2(dd * Ii.x * l, dd * Ii.y * l);
            rr[d] = ro[d] - rm[d];
        }
        const double2 mr = make_double2(m[0].x * rr[0] + m[1].x * rr[1] + m[2].x * rr[2],
                                        m[0].y * rr[0] + m[1].y * rr[1] + m[2].y * rr[2]);
        const double r2 = rr[0] * rr[0] + rr[1] * rr[1] + rr[2] * rr[2];
        const double R = sqrt(r2);
        double sn, cs;
        sincos(w_smue * R, &sn, &cs);
        const double2 g = make_double2(cs / R, -sn / R);
        for (int d = 0; d < 3; ++d) {
            const double2 v = make_double2(mr.x * rr[d] / r2 - m[d].x, mr.y * rr[d] / r2 - m[d].y);
            cmac(E[d], g, v);
        }
    }
    __shared__ double red[6][256];
    for (int d = 0; d < 3; ++d) { red[2 * d][threadIdx.x] = E[d].x; red[2 * d + 1][threadIdx.x] = E[d].y; }
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int q = 0; q < 6; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double s2 = 0;
        for (int d = 0; d < 3; ++d) {
            // E * (j facE)
            const double ex = -facE * red[2 * d + 1][0], ey = facE * red[2 * d][0];
            s2 += ex * ex + ey * ey;
        }
        sigma[a] = s2 * 4 * PI * (rzl * rzl) / den[a];
    }
}

int device_excitation(Ctx* c, const double* dirs, const double2* pols, double2 ctte, int nrhs, double2* b) {
    DevScope ds;
    double* ddirs = nullptr;
    double2* dpols = nullptr;
    CK(ds.alloc(&ddirs, 3 * (size_t)nrhs * sizeof(double)));
    CK(ds.alloc(&dpols, 3 * (size_t)nrhs * sizeof(double2)));
    CK(cudaMemcpyAsync(ddirs, dirs, 3 * (size_t)nrhs * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(dpols, pols, 3 * (size_t)nrhs * sizeof(double2), cudaMemcpyHostToDevice, c->stream));
    dim3 g((c->N + 127) / 128, nrhs);
    k_excitation<<<g, 128, 0, c->stream>>>(c->N, nrhs, ddirs, dpols, ctte, c->dp_coord, c->dt_baric, c->de_t,
                                           c->de_po, c->de_long, c->ph.w * c->ph.smue, b);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->stream));
    return MLF_OK;
}

// calc_RCS (modRCS.f90:109-153): observation radius from the edge-centre
// bounding box; calc_E uses the triangle centroids.  Angle a's currents are
// I + a istride and its polarisation pol + 3 (a pstride).
static int rcs_launch(Ctx* c, const double2* I, size_t istride, const double2* pol, int pstride, double2 ctte,
                      const double* th, const double* ph, int nang, double* sigma) {
    DevScope ds;
    const int N = c->N;
    const double* ec = c->e_centro.data();
    int lim[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 1; i < N; ++i) {
        const double* p = ec + 3 * i;
        if (p[0] > ec[3 * lim[0]]) lim[0] = i;
        if (p[0] < ec[3 * lim[1]]) lim[1] = i;
        if (p[1] > ec[3 * lim[2] + 1]) lim[2] = i;
        if (p[1] < ec[3 * lim[3] + 1]) lim[3] = i;
        if (p[2] > ec[3 * lim[4] + 2]) lim[4] = i;
        if (p[2] < ec[3 * lim[5] + 2]) lim[5] = i;
    }
    const double maxX = ec[3 * lim[0]], minX = ec[3 * lim[1]], maxY = ec[3 * lim[2] + 1],
                 minY = ec[3 * lim[3] + 1], maxZ = ec[3 * lim[4] + 2], minZ = ec[3 * lim[5] + 2];
    const double lambda = 2 * PI / (c->ph.w * std::sqrt(MU * EPSI));
    const double D = std::sqrt(((maxX - minX) * (maxX - minX)) + ((maxY - minY) * (maxY - minY)) +
                               ((maxZ - minZ) * (maxZ - minZ)));
    double rzl = 2 * (D * D) / lambda;
    if (50 * D > rzl) rzl = 50 * D;
    if (20 * lambda > rzl) rzl = 20 * lambda;
    rzl = rzl * 10;
    std::vector<double> den(nang, 0.0);
    for (int a = 0; a < nang; ++a)
        for (int d = 0; d < 3; ++d) {
            const double2 pv = pol[3 * (size_t)a * pstride + d];
            const double vx = pv.x * ctte.x - pv.y * ctte.y, vy = pv.x * ctte.y + pv.y * ctte.x;
            den[a] += vx * vx + vy * vy;
        }
    double *dth = nullptr, *dph = nullptr, *dsig = nullptr, *dden = nullptr;
    CK(ds.alloc(&dth, nang * sizeof(double)));
    CK(ds.alloc(&dph, nang * sizeof(double)));
    CK(ds.alloc(&dsig, nang * sizeof(double)));
    CK(ds.alloc(&dden, nang * sizeof(double)));
    CK(cudaMemcpyAsync(dth, th, nang * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(dph, ph, nang * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(dden, den.data(), nang * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    k_rcs<<<nang, 256, 0, c->stream>>>(N, c->dt_baric, c->de_t, c->de_long, I, istride, dth, dph,
                                       0.5 * (maxX + minX), 0.5 * (maxY + minY), 0.5 * (maxZ + minZ), rzl,
                                       c->ph.w * c->ph.smue, c->ph.w * MU / (4 * PI), dden, dsig);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(sigma, dsig, nang * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return MLF_OK;
}

// sigma(theta[a], phi[a]) of one current vector for nang bistatic angles
int device_rcs(Ctx* c, const double2* I, const double2* pol, double2 ctte, const double* th, const double* ph,
               int nang, double* sigma) {
    return rcs_launch(c, I, 0, pol, 0, ctte, th, ph, nang, sigma);
}

// one angle per column: column q (currents X + q ldx, polarisation pols + 3 q)
// at (th[q], ph[q]) -- the backscatter of a block of monostatic angles in one launch
int device_rcs_cols(Ctx* c, const double2* X, size_t ldx, int ncol, const double2* pols, double2 ctte,
                    const double* th, const double* ph, double* sigma) {
    return rcs_launch(c, X, ldx, pols, 1, ctte, th, ph, ncol, sigma);
}

}  // namespace mlf
