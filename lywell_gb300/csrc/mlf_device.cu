// Device side of the MLFMA solve on one GB300 (sm_103a).
//
// GB300 runs FP64 at about 1/64 of its FP32 rate, so the plain-FP64 matvec is
// bound by the FP64 pipe, not by HBM.  The kernels therefore keep every
// double-precision instruction that is not part of the algorithm's own
// arithmetic off the hot path: phase shifts between levels come from
// precomputed per-octant tables (no sincos), indices are integer, reductions
// use warp shuffles, and each complex multiply-add is four DFMA.
//
// Set-up kernels (once per context):
//   k_patterns      radiation patterns R (calcRad, modMLFMA.f90:584-703)
//   k_translation   T_n(k) per distinct displacement (calc_functransf,
//                   modMLFMA.f90:964-994), Legendre sum in IEEE round-to-nearest
//                   steps in the oracle's order
//   k_near          complex(4) near-field block (Zmn_MoM, modMoM.f90:85-128)
// Matvec kernels (MatxVec_MLFMA, modMLFMA.f90:1901-1946):
//   k_aggregate       leaf C = sum_n R_n x_n                  (:1805-1811)
//   k_interp_sep      parent C += shift * Interpolar(child C), as a theta
//                     pass then a phi pass (mlf_sep.cuh)       (:1818-1831)
//   k_translate       B = w * sum_far C_src T                  (:1838-1853)
//   k_anterp_sep      A = B + Anterpolar(shift* parent A|B), transposed
//                     phi pass then theta pass (mlf_sep.cuh)   (:1857-1897)
//   k_receive_near_d  y = fac sum conj(R) A + Znear x, near values in
//                     complex(8)                               (:1915-1942)
// fp64_matvec_launch issues these on given field buffers: the context's own
// (device_matvec) or the allocation-free entry point's fixed scratch
// (mlf_noalloc.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "mlf_internal.h"
#include "mlf_sep.cuh"
#include "mlf_zmn.cuh"

namespace mlf {

bool cuda_ok(Ctx* c, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    char buf[256];
    snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    c->err = buf;
    return false;
}

#define CK(call)                                   \
    do {                                           \
        if (!cuda_ok(c, (call), #call)) return MLF_E_CUDA; \
    } while (0)

template <class T>
static int upload(Ctx* c, T** dst, const std::vector<T>& v) {
    const size_t n = std::max<size_t>(v.size(), 1);
    CK(cudaMalloc((void**)dst, n * sizeof(T)));
    if (!v.empty()) CK(cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return MLF_OK;
}

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ void cmac(double2& acc, double2 a, double2 b) {
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(-a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(a.y, b.x, acc.y);
}

// ---------------------------------------------------------------------------
// set-up kernels
// ---------------------------------------------------------------------------

// R[j][p][k], j = position in the leaf-box-sorted basis list.
__global__ void k_patterns(int K, const int* __restrict__ bases, const int* __restrict__ box_of_sorted,
                           const double* __restrict__ centres, const double* __restrict__ t_baric,
                           const double* __restrict__ p_coord, const int* __restrict__ e_t,
                           const int* __restrict__ e_po, const double* __restrict__ e_long,
                           const double* __restrict__ kap, const double* __restrict__ ath,
                           const double* __restrict__ aph, double ka, int nchunk, double2* __restrict__ R) {
    const int j = blockIdx.x / nchunk;
    const int k = (blockIdx.x % nchunk) * blockDim.x + threadIdx.x;
    if (k >= K) return;
    const int n = bases[j];
    const double* C = centres + 3 * box_of_sorted[j];
    const double* bp = t_baric + 3 * e_t[2 * n];
    const double* vp = p_coord + 3 * e_po[2 * n];
    const double* bm = t_baric + 3 * e_t[2 * n + 1];
    const double* vm = p_coord + 3 * e_po[2 * n + 1];
    const double lon = e_long[n];
    const double* kk = kap + 3 * k;
    const double ap = ka * (kk[0] * (bp[0] - C[0]) + kk[1] * (bp[1] - C[1]) + kk[2] * (bp[2] - C[2]));
    const double am = ka * (kk[0] * (bm[0] - C[0]) + kk[1] * (bm[1] - C[1]) + kk[2] * (bm[2] - C[2]));
    double sp, cp, sm, cm;
    sincos(ap, &sp, &cp);
    sincos(am, &sm, &cm);
    double2 v0 = make_double2(0, 0), v1 = make_double2(0, 0);
    const double* at = ath + 3 * k;
    const double* af = aph + 3 * k;
    for (int d = 0; d < 3; ++d) {
        const double rp = bp[d] - vp[d], rm = vm[d] - bm[d];
        const double vr = ((cp * rp + cm * rm) * lon) * 0.5;
        const double vi = ((sp * rp + sm * rm) * lon) * 0.5;
        v0.x += vr * at[d]; v0.y += vi * at[d];
        v1.x += vr * af[d]; v1.y += vi * af[d];
    }
    R[(size_t)j * 2 * K + k] = v0;
    R[(size_t)j * 2 * K + K + k] = v1;
}

// T[t][k] = s * sum_{l<=Lt} c_l P_l(khat_k . u_t), c_l = (-j)^(l+1) (2l+1) h_l(kD).
// Legendre by the explicit binomial-square sum with round-to-nearest
// intrinsics (no contraction), or by the three-term recurrence.
__global__ void k_translation(int K, const double* __restrict__ kap, const double* __restrict__ u,
                              const int* __restrict__ Lt, const double2* __restrict__ coef, int ldc,
                              const double* __restrict__ binom2, int ldb, double scale, int mode,
                              double2* __restrict__ T) {
    const int t = blockIdx.y;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    const double* kk = kap + 3 * k;
    const double* ut = u + 3 * t;
    const double x = __dadd_rn(__dadd_rn(__dmul_rn(kk[0], ut[0]), __dmul_rn(kk[1], ut[1])),
                               __dmul_rn(kk[2], ut[2]));
    const int L = Lt[t];
    const double2* cf = coef + (size_t)t * ldc;
    double vr = 0., vi = 0.;
    if (mode == 1) {
        double pm = 1.0, pc = x;
        for (int l = 0; l <= L; ++l) {
            const double P = l == 0 ? 1.0 : pc;
            vr = __dadd_rn(vr, __dmul_rn(cf[l].x, P));
            vi = __dadd_rn(vi, __dmul_rn(cf[l].y, P));
            if (l >= 1) {
                const double nx = ((2.0 * l + 1.0) * x * pc - l * pm) / (l + 1.0);
                pm = pc;
                pc = nx;
            }
        }
    } else {
        double pa[128], pb[128];
        const double a = __dadd_rn(x, 1.0), b = __dadd_rn(x, -1.0);
        pa[0] = 1.0; pb[0] = 1.0;
        for (int q = 1; q <= L; ++q) { pa[q] = __dmul_rn(pa[q - 1], a); pb[q] = __dmul_rn(pb[q - 1], b); }
        for (int l = 0; l <= L; ++l) {
            const double* bn = binom2 + (size_t)l * ldb;
            double r = 0.;
            for (int i = 0; i <= l; ++i) r = __dadd_rn(r, __dmul_rn(__dmul_rn(bn[i], pa[l - i]), pb[i]));
            const double P = ldexp(r, -l);
            vr = __dadd_rn(vr, __dmul_rn(cf[l].x, P));
            vi = __dadd_rn(vi, __dmul_rn(cf[l].y, P));
        }
    }
    T[(size_t)t * K + k] = make_double2(__dmul_rn(vr, scale), __dmul_rn(vi, scale));
}

// One block per row m, threads over the row's near columns.
__global__ void k_near(const int* __restrict__ ia, const int* __restrict__ ja,
                       const double* __restrict__ t_baric, const double* __restrict__ t_baric_sub,
                       const double* __restrict__ p_coord, const int* __restrict__ e_t,
                       const int* __restrict__ e_po, const double* __restrict__ e_long, double w,
                       double w_smue, double c72, float2* __restrict__ Z) {
    const int m = blockIdx.x;
    const int beg = ia[m], end = ia[m + 1];
    for (int q = beg + threadIdx.x; q < end; q += blockDim.x) {
        const double2 v = zmn_mom(m, ja[q], t_baric, t_baric_sub, p_coord, e_t, e_po, e_long, w, w_smue, c72);
        Z[q] = make_float2((float)v.x, (float)v.y);
    }
}

// ---------------------------------------------------------------------------
// matvec kernels.  Fields carry nrhs columns: F[(box*nrhs + r)*2K + p*K + k].
// ---------------------------------------------------------------------------

// blockIdx.x = box*nrhs + r
__global__ void k_aggregate(int K, int nrhs, int ld, const int* __restrict__ box_ptr,
                            const int* __restrict__ perm, const double2* __restrict__ R,
                            const double2* __restrict__ x, double2* __restrict__ C) {
    const int b = blockIdx.x / nrhs, r = blockIdx.x % nrhs;
    const int j0 = box_ptr[b], j1 = box_ptr[b + 1];
    const double2* xr = x + (size_t)r * ld;
    for (int q = threadIdx.x; q < 2 * K; q += blockDim.x) {
        double2 acc = make_double2(0, 0);
        for (int j = j0; j < j1; ++j) cmac(acc, R[(size_t)j * 2 * K + q], xr[perm[j]]);
        C[((size_t)b * nrhs + r) * 2 * K + q] = acc;
    }
}

// blockIdx.x = (box*nrhs + r)*nchunk + chunk
__global__ void k_translate(int K, int nrhs, int nchunk, const int* __restrict__ far_ptr,
                            const int* __restrict__ far_src, const int* __restrict__ far_tid,
                            const double2* __restrict__ T, const double* __restrict__ wq,
                            const double2* __restrict__ C, double2* __restrict__ B) {
    const int chunk = blockIdx.x % nchunk;
    const int br = blockIdx.x / nchunk;
    const int b = br / nrhs, r = br % nrhs;
    const int q = chunk * blockDim.x + threadIdx.x;
    if (q >= 2 * K) return;
    const int k = q >= K ? q - K : q;
    double2 acc = make_double2(0, 0);
    const int f1 = far_ptr[b + 1];
    for (int f = far_ptr[b]; f < f1; ++f) {
        const double2 cs = C[((size_t)far_src[f] * nrhs + r) * 2 * K + q];
        cmac(acc, cs, T[(size_t)far_tid[f] * K + k]);
    }
    const double wk = wq[k];
    B[((size_t)b * nrhs + r) * 2 * K + q] = make_double2(acc.x * wk, acc.y * wk);
}

// One warp per (sorted basis j, rhs): y[perm[j]] = fac * sum conj(R_j) A_box
// + sum_near Z x, with the near field held as complex(8): the complex(4)
// values of the reference converted once at set-up, so the SpMV spends no
// FP64-pipe slots on float -> double conversions.
__global__ void k_receive_near_d(int K, int N, int nrhs, int ld, const int* __restrict__ perm,
                                 const int* __restrict__ box_of_sorted, const double2* __restrict__ R,
                                 const double2* __restrict__ A, const int* __restrict__ ia,
                                 const int* __restrict__ ja, const double2* __restrict__ Zd,
                                 const double2* __restrict__ x, double facy, double2* __restrict__ y) {
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (gw >= N * nrhs) return;
    const int j = gw / nrhs, r = gw % nrhs;
    const int n = perm[j], b = box_of_sorted[j];
    const double2* Rj = R + (size_t)j * 2 * K;
    const double2* Ab = A + ((size_t)b * nrhs + r) * 2 * K;
    double sr = 0, si = 0;
    for (int q = lane; q < 2 * K; q += 32) {
        const double2 a = Rj[q], v = Ab[q];
        sr = fma(a.x, v.x, sr); sr = fma(a.y, v.y, sr);
        si = fma(a.x, v.y, si); si = fma(-a.y, v.x, si);
    }
    const double2* xr = x + (size_t)r * ld;
    double nr = 0, ni = 0;
    for (int q = ia[n] + lane; q < ia[n + 1]; q += 32) {
        const double2 z = Zd[q];
        const double2 xv = xr[ja[q]];
        nr = fma(xv.x, z.x, nr); nr = fma(-xv.y, z.y, nr);
        ni = fma(xv.x, z.y, ni); ni = fma(xv.y, z.x, ni);
    }
    // combine before the reduction: t = j*facy*s + near
    double tr = fma(-facy, si, nr), ti = fma(facy, sr, ni);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        tr += __shfl_xor_sync(0xffffffff, tr, o);
        ti += __shfl_xor_sync(0xffffffff, ti, o);
    }
    if (lane == 0) y[(size_t)r * ld + n] = make_double2(tr, ti);
}

__global__ void k_f2d(size_t n, const float2* __restrict__ a, double2* __restrict__ b) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        b[i] = make_double2((double)a[i].x, (double)a[i].y);
}

// ---------------------------------------------------------------------------
// set-up driver
// ---------------------------------------------------------------------------

static int launch_check(Ctx* c, const char* what) {
    return cuda_ok(c, cudaGetLastError(), what) ? MLF_OK : MLF_E_CUDA;
}

int ensure_fields(Ctx* c, int nrhs) {
    for (int n = 3; n <= c->nlev; ++n) {
        Level& L = c->lv[n];
        if (L.fcap >= nrhs) continue;
        cudaFree(L.dC); cudaFree(L.dB); cudaFree(L.dA);
        L.dC = L.dB = L.dA = nullptr;
        const size_t fsz = (size_t)L.nb * nrhs * 2 * L.K;
        CK(cudaMalloc(&L.dC, fsz * sizeof(double2)));
        CK(cudaMalloc(&L.dB, fsz * sizeof(double2)));
        CK(cudaMalloc(&L.dA, fsz * sizeof(double2)));
        L.fcap = nrhs;
    }
    return MLF_OK;
}

int fetch_near_values(Ctx* c, std::vector<float2>& out) {
    out.resize(c->nnz);
    CK(cudaMemcpy(out.data(), c->dZ, c->nnz * sizeof(float2), cudaMemcpyDeviceToHost));
    return MLF_OK;
}

// Replace the complex(4) near-field values (the reference's public
// Zesparcida_MLFMA, which its host may overwrite before crear_precond) and
// drop everything derived from them: the complex(8) copy is rebuilt, the
// box-pair blocks are rebuilt on their next use, and the ILU / neighbourhood
// preconditioners must be built again.
int device_set_near(Ctx* c, const float2* host_vals) {
    CK(cudaMemcpyAsync(c->dZ, host_vals, c->nnz * sizeof(float2), cudaMemcpyHostToDevice, c->stream));
    k_f2d<<<4096, 256, 0, c->stream>>>((size_t)c->nnz, c->dZ, c->dZd);
    int st;
    if ((st = launch_check(c, "k_f2d"))) return st;
    CK(cudaStreamSynchronize(c->stream));
    near_blocks_free(c);
    c->ilu_ok = 0;
    c->nearinv_ok = 0;
    c->nearinv_own = 0;
    c->learned = 0;
    return MLF_OK;
}

int need_tree(Ctx* c) {
    if (!c->dense) return 0;
    c->err = "this call needs the MLFMA octree; the context holds the dense MoM operator";
    return 1;
}

int upload_geometry(Ctx* c) {
    int st;
    if ((st = upload(c, &c->dp_coord, c->p_coord))) return st;
    if ((st = upload(c, &c->dt_baric, c->t_baric))) return st;
    if ((st = upload(c, &c->dt_baric_sub, c->t_baric_sub))) return st;
    if ((st = upload(c, &c->de_long, c->e_long))) return st;
    if ((st = upload(c, &c->de_centro, c->e_centro))) return st;
    if ((st = upload(c, &c->de_t, c->e_t))) return st;
    if ((st = upload(c, &c->de_po, c->e_po))) return st;
    return MLF_OK;
}

int device_setup(Ctx* c) {
    CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    for (int i = 0; i < 8; ++i) CK(cudaEventCreate(&c->ev[i]));
    const int nl = c->nlev;
    const int N = c->N;
    int st;
    if ((st = upload_geometry(c))) return st;
    Level& leaf = c->lv[nl];
    std::vector<int> box_of_sorted(N);
    for (int b = 0; b < leaf.nb; ++b)
        for (int j = c->box_ptr[b]; j < c->box_ptr[b + 1]; ++j) box_of_sorted[j] = b;
    if ((st = upload(c, &c->dperm, c->box_bases))) return st;
    if ((st = upload(c, &c->dbox_ptr, c->box_ptr))) return st;
    if ((st = upload(c, &c->dbox_of_sorted, box_of_sorted))) return st;
    if ((st = upload(c, &c->dia, c->ia))) return st;
    if ((st = upload(c, &c->dja, c->ja))) return st;
    if ((st = ensure_fields(c, 1))) return st;
    for (int n = 3; n <= nl; ++n) {
        Level& L = c->lv[n];
        if ((st = upload(c, &L.dwq, L.wq))) return st;
        if ((st = upload(c, &L.dkap, L.kap))) return st;
        if ((st = upload(c, &L.dath, L.ath))) return st;
        if ((st = upload(c, &L.daph, L.aph))) return st;
        if ((st = upload(c, &L.dcentre, L.centre))) return st;
        if ((st = upload(c, &L.dfar_ptr, L.far_ptr))) return st;
        if ((st = upload(c, &L.dfar_src, L.far_src))) return st;
        if ((st = upload(c, &L.dfar_tid, L.far_tid))) return st;
        if ((st = upload(c, &L.dparent, L.parent))) return st;
        if ((st = upload(c, &L.doctant, L.octant))) return st;
        if (n < nl) {
            if ((st = upload(c, &L.dchild_ptr, L.child_ptr))) return st;
            if ((st = upload(c, &L.dsth, L.sth))) return st;
            if ((st = upload(c, &L.dsph, L.sph))) return st;
            if ((st = upload(c, &L.dwth, L.wth))) return st;
            if ((st = upload(c, &L.dwph, L.wph))) return st;
            if ((st = upload(c, &L.dthT_ptr, L.thT_ptr))) return st;
            if ((st = upload(c, &L.dthT_row, L.thT_row))) return st;
            if ((st = upload(c, &L.dthT_w, L.thT_w))) return st;
            if ((st = upload(c, &L.dphT_ptr, L.phT_ptr))) return st;
            if ((st = upload(c, &L.dphT_row, L.phT_row))) return st;
            if ((st = upload(c, &L.dphT_w, L.phT_w))) return st;
            // phase tables of this (parent) level for the 8 child octants:
            // exp(+j k khat . r), r = (+-q, +-q, +-q), q = side/4
            std::vector<double2> sh(8 * (size_t)L.K);
            static const int sx[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
            static const int sy[8] = {-1, 1, -1, 1, -1, 1, -1, 1};
            static const int sz[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
            const double q = L.side / 4., k0 = (2. * PI) / c->ph.lambda;
            for (int o = 0; o < 8; ++o)
                for (int m = 0; m < L.K; ++m) {
                    const double* kk = &L.kap[3 * (size_t)m];
                    const double kr = kk[0] * (sx[o] * q) + kk[1] * (sy[o] * q) + kk[2] * (sz[o] * q);
                    const double a = k0 * kr;
                    sh[(size_t)o * L.K + m] = make_double2(std::cos(a), std::sin(a));
                }
            if ((st = upload(c, &L.dshift, sh))) return st;
        }
    }
    // translation tables
    int Lmax = 0;
    for (int n = 3; n <= nl; ++n) Lmax = std::max(Lmax, c->lv[n].L);
    const int mode = (c->flags & MLF_FLAG_LEGENDRE_RECURRENCE) ? 1 : 0;
    if (Lmax > 127 && mode == 0) {
        c->err = "explicit Legendre sum limited to L <= 127; use MLF_FLAG_LEGENDRE_RECURRENCE";
        return MLF_E_ARG;
    }
    std::vector<double> b2;
    binomial_squares(Lmax, b2);
    double* db2 = nullptr;
    if ((st = upload(c, &db2, b2))) return st;
    for (int n = 3; n <= nl; ++n) {
        Level& L = c->lv[n];
        const int nt = L.ntrans;
        const int ldc = L.L + 1;
        std::vector<double> u(3 * (size_t)std::max(nt, 1));
        std::vector<int> Lt(std::max(nt, 1));
        std::vector<double2> coef((size_t)std::max(nt, 1) * ldc, make_double2(0, 0));
        std::vector<double> jb(L.L + 2), yb(L.L + 2);
        for (int t = 0; t < nt; ++t) {
            const double* rab = &L.rab[3 * (size_t)t];
            const double mod = std::sqrt(rab[0] * rab[0] + rab[1] * rab[1] + rab[2] * rab[2]);
            const double kD = (2. * PI / c->ph.lambda) * mod;
            int Ltrue = L.L;
            const int kDint = (int)kD;
            if (kDint < Ltrue) Ltrue = kDint;   // multipole clipping (modMLFMA.f90:976-982)
            Lt[t] = Ltrue;
            for (int d = 0; d < 3; ++d) u[3 * t + d] = rab[d] / mod;
            sph_bessel(Ltrue, kD, jb.data(), yb.data());
            for (int l = 0; l <= Ltrue; ++l) {
                // ((-j)^(l+1) (2l+1)) * (j_l - j y_l): one factor component is zero
                const double f = 2. * l + 1;
                const double hr = jb[l], hi = -yb[l];
                double ar = 0, ai = 0;
                switch ((l + 1) & 3) {
                    case 0: ar = f; break;
                    case 1: ai = -f; break;
                    case 2: ar = -f; break;
                    default: ai = f; break;
                }
                coef[(size_t)t * ldc + l] = make_double2(ar * hr - ai * hi, ar * hi + ai * hr);
            }
        }
        double* du = nullptr;
        int* dLt = nullptr;
        double2* dcoef = nullptr;
        if ((st = upload(c, &du, u))) return st;
        if ((st = upload(c, &dLt, Lt))) return st;
        if ((st = upload(c, &dcoef, coef))) return st;
        CK(cudaMalloc(&L.dT, std::max<size_t>((size_t)nt * L.K, 1) * sizeof(double2)));
        const double scale = (2. * PI / c->ph.lambda) / (4. * PI);
        for (int t0 = 0; t0 < nt; t0 += 65535) {   // grid.y limit (single-level FMM grids have many vectors)
            const int cnt = std::min(65535, nt - t0);
            dim3 grid((L.K + 127) / 128, cnt);
            k_translation<<<grid, 128, 0, c->stream>>>(L.K, L.dkap, du + 3 * (size_t)t0, dLt + t0,
                                                       dcoef + (size_t)t0 * ldc, ldc, db2, Lmax + 1, scale, mode,
                                                       L.dT + (size_t)t0 * L.K);
            if ((st = launch_check(c, "k_translation"))) return st;
        }
        CK(cudaStreamSynchronize(c->stream));
        cudaFree(du);
        cudaFree(dLt);
        cudaFree(dcoef);
    }
    cudaFree(db2);
    // radiation patterns in box order
    CK(cudaMalloc(&c->dR, (size_t)N * 2 * leaf.K * sizeof(double2)));
    {
        const int nch = (leaf.K + 127) / 128;
        k_patterns<<<N * nch, 128, 0, c->stream>>>(leaf.K, c->dperm, c->dbox_of_sorted, leaf.dcentre,
                                                   c->dt_baric, c->dp_coord, c->de_t, c->de_po, c->de_long,
                                                   leaf.dkap, leaf.dath, leaf.daph, (2. * PI) / c->ph.lambda,
                                                   nch, c->dR);
        if ((st = launch_check(c, "k_patterns"))) return st;
    }
    // near field
    CK(cudaMalloc(&c->dZ, std::max<long long>(c->nnz, 1) * sizeof(float2)));
    {
        const double c72 = (double)(1.0f / 72.0f);
        k_near<<<N, 128, 0, c->stream>>>(c->dia, c->dja, c->dt_baric, c->dt_baric_sub, c->dp_coord,
                                         c->de_t, c->de_po, c->de_long, c->ph.w, c->ph.w * c->ph.smue,
                                         c72, c->dZ);
        if ((st = launch_check(c, "k_near"))) return st;
        CK(cudaMalloc(&c->dZd, std::max<long long>(c->nnz, 1) * sizeof(double2)));
        k_f2d<<<4096, 256, 0, c->stream>>>((size_t)c->nnz, c->dZ, c->dZd);
        if ((st = launch_check(c, "k_f2d"))) return st;
    }
    CK(cudaStreamSynchronize(c->stream));
    return MLF_OK;
}

// ---------------------------------------------------------------------------
// matvec driver
// ---------------------------------------------------------------------------

static inline int chunks(int n, int bd) { return (n + bd - 1) / bd; }

// The FP64 operator's launches on the given field buffers (level n: Cf[n],
// Bf[n], Af[n], each double2[nb_n][nrhs][2][K_n]).  device_matvec passes the
// context's buffers; mlf_matvec_device_noalloc passes buffers carved from its
// fixed scratch, so both run the same kernels in the same order.  ev: six
// events recorded between the stages (profiling), or nullptr.
int fp64_matvec_launch(Ctx* c, const double2* x, double2* y, int nrhs, int ld, cudaStream_t s,
                       double2* const* Cf, double2* const* Bf, double2* const* Af, cudaEvent_t* ev) {
    const int nl = c->nlev;
    Level& leaf = c->lv[nl];
    if (ev) cudaEventRecord(ev[0], s);
    k_aggregate<<<leaf.nb * nrhs, 256, 0, s>>>(leaf.K, nrhs, ld, c->dbox_ptr, c->dperm, c->dR, x, Cf[nl]);
    if (ev) cudaEventRecord(ev[1], s);
    for (int n = nl; n >= 4; --n) {
        Level& Lc = c->lv[n];
        Level& Lp = c->lv[n - 1];
        const int nslab = chunks(Lp.L, SEP_SLAB);
        const size_t smem = (size_t)SEP_SLAB * 2 * (Lc.L + Lp.L) * sizeof(double2);   // child rows + parent slab
        k_interp_sep<double2, 1><<<Lp.nb * nrhs * 2 * nslab, 256, smem, s>>>(
            Lp.L, Lc.L, nrhs, nslab, Lp.dchild_ptr, Lc.doctant, Lp.dsth, Lp.dwth, Lp.dsph, Lp.dwph, Lp.dshift,
            Cf[n], Cf[n - 1]);
    }
    if (ev) cudaEventRecord(ev[2], s);
    for (int n = 3; n <= nl; ++n) {
        Level& L = c->lv[n];
        const int bd = 128, nch = chunks(2 * L.K, bd);
        k_translate<<<L.nb * nrhs * nch, bd, 0, s>>>(L.K, nrhs, nch, L.dfar_ptr, L.dfar_src, L.dfar_tid,
                                                     L.dT, L.dwq, Cf[n], Bf[n]);
    }
    if (ev) cudaEventRecord(ev[3], s);
    for (int n = 4; n <= nl; ++n) {
        Level& Lc = c->lv[n];
        Level& Lp = c->lv[n - 1];
        const double2* Psrc = (n == 4) ? Bf[n - 1] : Af[n - 1];
        const size_t smem = ((size_t)Lp.K + (size_t)Lp.L * 2 * Lc.L) * sizeof(double2);
        k_anterp_sep<double2, 1><<<Lc.nb * nrhs * 2, 256, smem, s>>>(
            Lp.L, Lc.L, nrhs, Lc.dparent, Lc.doctant, Lp.dthT_ptr, Lp.dthT_row, Lp.dthT_w, Lp.dphT_ptr,
            Lp.dphT_row, Lp.dphT_w, Lp.dshift, Psrc, Bf[n], Af[n]);
    }
    if (ev) cudaEventRecord(ev[4], s);
    {
        const int warps = c->N * nrhs;
        const double facy = c->ph.w * MU / (4. * PI);
        k_receive_near_d<<<chunks(warps * 32, 256), 256, 0, s>>>(leaf.K, c->N, nrhs, ld, c->dperm,
                                                                  c->dbox_of_sorted, c->dR,
                                                                  nl == 3 ? Bf[nl] : Af[nl], c->dia,
                                                                  c->dja, c->dZd, x, facy, y);
    }
    if (ev) cudaEventRecord(ev[5], s);
    return launch_check(c, "matvec");
}

int device_matvec(Ctx* c, const double2* x, double2* y, int nrhs, int ld, cudaStream_t s) {
    if (c->dense) return dense_matvec(c, x, y, nrhs, ld, s);
    if (c->mv_prec == 1) return device_matvec32(c, x, y, nrhs, ld, s);
    int st;
    if ((st = ensure_fields(c, nrhs))) return st;
    c->last_nrhs = nrhs;
    double2* Cf[32] = {nullptr};
    double2* Bf[32] = {nullptr};
    double2* Af[32] = {nullptr};
    for (int n = 3; n <= c->nlev; ++n) {
        Cf[n] = c->lv[n].dC;
        Bf[n] = c->lv[n].dB;
        Af[n] = c->lv[n].dA;
    }
    const bool prof = c->profiling != 0;
    if ((st = fp64_matvec_launch(c, x, y, nrhs, ld, s, Cf, Bf, Af, prof ? c->ev : nullptr))) return st;
    if (prof) {
        CK(cudaEventSynchronize(c->ev[5]));
        for (int i = 0; i < 5; ++i) cudaEventElapsedTime(&c->stage_ms[i], c->ev[i], c->ev[i + 1]);
    }
    return MLF_OK;
}

// anterpolation smem: the largest parent grid decides; opt in above 48 KB
int configure_kernels(Ctx* c) {
    size_t mx2 = 0, mx3 = 0;
    for (int n = 3; n < c->nlev; ++n) {
        mx2 = std::max(mx2, ((size_t)c->lv[n].K + (size_t)c->lv[n].L * 2 * c->lv[n + 1].L) * sizeof(double2));
        mx3 = std::max(mx3, (size_t)SEP_SLAB * 2 * (c->lv[n + 1].L + c->lv[n].L) * sizeof(double2));
    }
    int optin = 0;
    CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->dev));
    if (mx2 > (size_t)optin || mx3 > (size_t)optin) {
        c->err = "parent sampling grid too large for the shared-memory interpolation stages";
        return MLF_E_ARG;
    }
    // The limit is a property of the kernel, shared by every context in the
    // process: raise it to the device maximum (what a launch actually uses is
    // its own dynamic size), never to one context's need, which would break
    // the launches of an earlier context with larger grids.
    CK(cudaFuncSetAttribute(k_anterp_sep<double2, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    CK(cudaFuncSetAttribute(k_interp_sep<double2, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    return MLF_OK;
}

void device_free(Ctx* c) {
    auto F = [](void* p) { if (p) cudaFree(p); };
    for (int n = 1; n <= c->nlev && n < 32; ++n) {
        Level& L = c->lv[n];
        F(L.dC); F(L.dB); F(L.dA); F(L.dT); F(L.dwq); F(L.dfar_ptr); F(L.dfar_src); F(L.dfar_tid);
        F(L.dshift);
        F(L.dchild_ptr); F(L.dparent); F(L.doctant); F(L.dkap); F(L.dath); F(L.daph); F(L.dcentre);
        F(L.dsth); F(L.dsph); F(L.dwth); F(L.dwph); F(L.dthT_ptr); F(L.dthT_row); F(L.dthT_w); F(L.dphT_ptr);
        F(L.dphT_row); F(L.dphT_w);
    }
    F(c->dR); F(c->dperm); F(c->dbox_ptr); F(c->dbox_of_sorted); F(c->dia); F(c->dja); F(c->dZ);
    F(c->dp_coord); F(c->dt_baric); F(c->dt_baric_sub); F(c->de_long); F(c->de_centro); F(c->de_t);
    F(c->de_po); F(c->dalu); F(c->djlu); F(c->dju); F(c->dlvl_rows_f); F(c->dlvl_rows_b);
    F(c->dwork); F(c->dscal); F(c->dflags); F(c->dx_io); F(c->dy_io); F(c->dMinv); F(c->dZd); F(c->dboff); F(c->dMinv32); F(c->dpre_xs); F(c->dZdense); F(c->dMinv_base);
    mixed_free(c);
    near_blocks_free(c);
    for (int i = 0; i < 8; ++i)
        if (c->ev[i]) cudaEventDestroy(c->ev[i]);
    for (int i = 0; i < 4; ++i)
        if (c->sev[i]) cudaEventDestroy(c->sev[i]);
    if (c->stream) cudaStreamDestroy(c->stream);
}

}  // namespace mlf
