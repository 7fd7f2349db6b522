// Mixed-precision solve: FP32 MLFMA matvec inside an FP64 iterative-refinement
// loop.  (An addition of this library: the reference runs its whole matvec
// with complex(8) fields, modMLFMA.f90:1783-1946.)
//
// FP32 operator: radiation patterns, translation tables, interpolation and
// anterpolation weights, phase-shift tables and all C/B/A fields are float;
// every stage accumulates in FP32 on the CUDA cores, which GB300 runs 64x
// faster than FP64; the near field is the reference's complex(4) block
// itself.  Input and output vectors stay complex(8).
//
// Refinement (mode 1 of mlf_solve): r = b - A64 x in FP64; one restart cycle
// of right-preconditioned GMRES(m) solves A d = r with an FP32 inner loop
// (operator, preconditioner, Krylov basis and Gram-Schmidt in float) until its
// residual estimate drops below inner_tol ||b|| or m steps; x += M^-1 V y,
// accumulated in FP64; stop when the FP64 residual ||b - A64 x|| < tol ||b||.
// The FP64 residual decides, so the result meets the same stopping test as
// the plain FP64 solve.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <memory>
#include <type_traits>
#include <vector>

#include "mlf_internal.h"
#include "mlf_sep.cuh"

namespace mlf {

#define CK(call)                                             \
    do {                                                     \
        if (!cuda_ok(c, (call), #call)) return MLF_E_CUDA;   \
    } while (0)

__device__ __forceinline__ void fmac(float2& acc, float2 a, float2 b) {
    acc.x = fmaf(a.x, b.x, acc.x);
    acc.x = fmaf(-a.y, b.y, acc.x);
    acc.y = fmaf(a.x, b.y, acc.y);
    acc.y = fmaf(a.y, b.x, acc.y);
}

// Krylov basis storage: FP32, or FP16 scaled by s = sqrt(N) on store (a unit
// column has every entry within sqrt(N), inside FP16's range) and by 1/s on
// load.  Arithmetic stays FP32 either way.
__device__ __forceinline__ float2 bload(const float2* p, float) { return *p; }
__device__ __forceinline__ float2 bload(const __half2* p, float s) {
    const float2 v = __half22float2(*p);
    return make_float2(v.x * s, v.y * s);
}
__device__ __forceinline__ void bstore(float2* p, float2 v, float) { *p = v; }
__device__ __forceinline__ void bstore(__half2* p, float2 v, float s) { *p = __floats2half2_rn(v.x * s, v.y * s); }

__global__ void k32_from64(size_t n, const double2* __restrict__ a, float2* __restrict__ b) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        b[i] = make_float2((float)a[i].x, (float)a[i].y);
}

// x (FP64, ld) -> packed FP32 columns
__global__ void k32_pack_x(int N, int nrhs, int ld, const double2* __restrict__ x, float2* __restrict__ xf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = blockIdx.y;
    if (i < N) {
        const double2 v = x[(size_t)r * ld + i];
        xf[(size_t)r * N + i] = make_float2((float)v.x, (float)v.y);
    }
}

__global__ void k32_aggregate(int K, int nrhs, int N, const int* __restrict__ box_ptr, const int* __restrict__ perm,
                              const float2* __restrict__ R, const float2* __restrict__ xf, float2* __restrict__ C) {
    const int b = blockIdx.x / nrhs, r = blockIdx.x % nrhs;
    const int j0 = box_ptr[b], j1 = box_ptr[b + 1];
    const float2* xr = xf + (size_t)r * N;
    for (int q = threadIdx.x; q < 2 * K; q += blockDim.x) {
        float2 acc = make_float2(0.f, 0.f);
        for (int j = j0; j < j1; ++j) fmac(acc, R[(size_t)j * 2 * K + q], xr[perm[j]]);
        C[((size_t)b * nrhs + r) * 2 * K + q] = acc;
    }
}

// B(:, col, box) = wq * sum over the far boxes of T_tid * C(:, col, src)
// (llenar_campoCyB, modMLFMA.f90:1838-1852) for both polarisations and columns
// [c0, c0 + NR): each thread owns one sample k, so each translation value is
// read once per 2 NR products.
template <int NR>
__global__ void k32_translate(int K, int nrhs, int nchunk, const int* __restrict__ far_ptr,
                              const int* __restrict__ far_src, const int* __restrict__ far_tid,
                              const float2* __restrict__ T, const float* __restrict__ wq,
                              const float2* __restrict__ C, float2* __restrict__ B) {
    const int chunk = blockIdx.x % nchunk;
    const int b = blockIdx.x / nchunk;
    const int c0 = blockIdx.y * NR;
    const int k = chunk * blockDim.x + threadIdx.x;
    if (k >= K) return;
    const size_t K2 = 2 * (size_t)K;
    float2 a0[NR], a1[NR];
#pragma unroll
    for (int u = 0; u < NR; ++u) a0[u] = a1[u] = make_float2(0.f, 0.f);
    const int f1 = far_ptr[b + 1];
    for (int f = far_ptr[b]; f < f1; ++f) {
        const float2 t = T[(size_t)far_tid[f] * K + k];
        const float2* cs = C + ((size_t)far_src[f] * nrhs + c0) * K2 + k;
#pragma unroll
        for (int u = 0; u < NR; ++u) {
            if (c0 + u < nrhs) {
                fmac(a0[u], cs[u * K2], t);
                fmac(a1[u], cs[u * K2 + K], t);
            }
        }
    }
    const float wk = wq[k];
    float2* bo = B + ((size_t)b * nrhs + c0) * K2 + k;
#pragma unroll
    for (int u = 0; u < NR; ++u) {
        if (c0 + u < nrhs) {
            bo[u * K2] = make_float2(a0[u].x * wk, a0[u].y * wk);
            bo[u * K2 + K] = make_float2(a1[u].x * wk, a1[u].y * wk);
        }
    }
}

// The same sums for a group of G consecutive boxes (G i .. G i + G - 1, in
// depth-first order and mostly siblings) over the merged list of their far
// boxes: each source value read from L2 serves every box of the group that
// has it, so the stage's L2 traffic, which bounds it, drops.  One thread per
// sample k, both polarisations, NR columns and the G boxes in registers.
template <int NR, int G>
__global__ void k32_translate_grp(int K, int nb, int nrhs, int nchunk, const int* __restrict__ gptr,
                                  const int* __restrict__ gsrc, const int* __restrict__ gtid,
                                  const float2* __restrict__ T, const float* __restrict__ wq,
                                  const float2* __restrict__ C, float2* __restrict__ B) {
    const int chunk = blockIdx.x % nchunk;
    const int gr = blockIdx.x / nchunk;
    const int c0 = blockIdx.y * NR;
    const int k = chunk * blockDim.x + threadIdx.x;
    if (k >= K) return;
    const size_t K2 = 2 * (size_t)K;
    float2 acc[G][2][NR];
#pragma unroll
    for (int h = 0; h < G; ++h)
#pragma unroll
        for (int u = 0; u < NR; ++u) acc[h][0][u] = acc[h][1][u] = make_float2(0.f, 0.f);
    const int e1 = gptr[gr + 1];
    for (int e = gptr[gr]; e < e1; ++e) {
        int t[G];   // the same for the whole CTA: uniform branches
        if (G == 4) {
            const int4 q = reinterpret_cast<const int4*>(gtid)[e];
            t[0] = q.x; t[1] = q.y; t[2 % G] = q.z; t[3 % G] = q.w;
        } else {
            const int2 q = reinterpret_cast<const int2*>(gtid)[e];
            t[0] = q.x; t[1 % G] = q.y;
        }
        const float2* cs = C + ((size_t)gsrc[e] * nrhs + c0) * K2 + k;
        float2 tv[G];
#pragma unroll
        for (int h = 0; h < G; ++h) tv[h] = t[h] >= 0 ? T[(size_t)t[h] * K + k] : make_float2(0.f, 0.f);
#pragma unroll
        for (int u = 0; u < NR; ++u) {
            if (c0 + u < nrhs) {
                const float2 p = cs[u * K2], q = cs[u * K2 + K];
#pragma unroll
                for (int h = 0; h < G; ++h)
                    if (t[h] >= 0) { fmac(acc[h][0][u], p, tv[h]); fmac(acc[h][1][u], q, tv[h]); }
            }
        }
    }
    const float wk = wq[k];
#pragma unroll
    for (int h = 0; h < G; ++h) {
        const int b = G * gr + h;
        if (b >= nb) break;
        float2* bo = B + ((size_t)b * nrhs + c0) * K2 + k;
#pragma unroll
        for (int u = 0; u < NR; ++u) {
            if (c0 + u < nrhs) {
                bo[u * K2] = make_float2(acc[h][0][u].x * wk, acc[h][0][u].y * wk);
                bo[u * K2 + K] = make_float2(acc[h][1][u].x * wk, acc[h][1][u].y * wk);
            }
        }
    }
}

__global__ void k32_receive_near(int K, int N, int nrhs, int ld, const int* __restrict__ perm,
                                 const int* __restrict__ box_of_sorted, const float2* __restrict__ R,
                                 const float2* __restrict__ A, const int* __restrict__ ia, const int* __restrict__ ja,
                                 const float2* __restrict__ Z, const float2* __restrict__ xf, float facy,
                                 double2* __restrict__ y) {
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (gw >= N * nrhs) return;
    const int j = gw / nrhs, r = gw % nrhs;
    const int n = perm[j], b = box_of_sorted[j];
    const float2* Rj = R + (size_t)j * 2 * K;
    const float2* Ab = A + ((size_t)b * nrhs + r) * 2 * K;
    float sr = 0.f, si = 0.f;
    for (int q = lane; q < 2 * K; q += 32) {
        const float2 a = Rj[q], v = Ab[q];
        sr = fmaf(a.x, v.x, sr); sr = fmaf(a.y, v.y, sr);
        si = fmaf(a.x, v.y, si); si = fmaf(-a.y, v.x, si);
    }
    const float2* xr = xf + (size_t)r * N;
    float nr = 0.f, ni = 0.f;
    for (int q = ia[n] + lane; q < ia[n + 1]; q += 32) {
        const float2 z = Z[q];
        const float2 xv = xr[ja[q]];
        nr = fmaf(xv.x, z.x, nr); nr = fmaf(-xv.y, z.y, nr);
        ni = fmaf(xv.x, z.y, ni); ni = fmaf(xv.y, z.x, ni);
    }
    float tr = fmaf(-facy, si, nr), ti = fmaf(facy, sr, ni);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        tr += __shfl_xor_sync(0xffffffff, tr, o);
        ti += __shfl_xor_sync(0xffffffff, ti, o);
    }
    if (lane == 0) y[(size_t)r * ld + n] = make_double2((double)tr, (double)ti);
}

// ---------------------------------------------------------------------------

static int up32(Ctx* c, float** dst, const std::vector<double>& v) {
    std::vector<float> f(v.begin(), v.end());
    CK(cudaMalloc(dst, std::max<size_t>(f.size(), 1) * sizeof(float)));
    if (!f.empty()) CK(cudaMemcpy(*dst, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice));
    return MLF_OK;
}

static int conv32(Ctx* c, float2** dst, const double2* src, size_t n) {
    CK(cudaMalloc(dst, std::max<size_t>(n, 1) * sizeof(float2)));
    if (n) k32_from64<<<(unsigned)std::min<size_t>((n + 255) / 256, 65535), 256, 0, c->stream>>>(n, src, *dst);
    CK(cudaGetLastError());
    return MLF_OK;
}

// Merged far lists of the box groups (G i .. G i + G - 1) of one level,
// sources ascending, with each source's translation index per box (-1 where
// it is not far from that box).
static int group_lists(Ctx* c, const Level& L, int G, Mixed32::Lv::Grp& M) {
    const int ng = (L.nb + G - 1) / G;
    std::vector<int> gptr(ng + 1, 0), gsrc, gtid;
    std::vector<std::pair<int, int>> ent;   // (source, box within the group), then the translation
    std::vector<int> etid;
    for (int g = 0; g < ng; ++g) {
        ent.clear();
        etid.clear();
        for (int h = 0; h < G && G * g + h < L.nb; ++h) {
            const int b = G * g + h;
            for (int f = L.far_ptr[b]; f < L.far_ptr[b + 1]; ++f) ent.push_back({L.far_src[f], (h << 20) | (int)etid.size()}), etid.push_back(L.far_tid[f]);
        }
        std::sort(ent.begin(), ent.end());
        for (size_t q = 0; q < ent.size(); ++q) {
            const int h = ent[q].second >> 20, t = etid[ent[q].second & 0xfffff];
            if (q == 0 || ent[q].first != ent[q - 1].first) {
                gsrc.push_back(ent[q].first);
                gtid.insert(gtid.end(), G, -1);
            }
            gtid[gtid.size() - G + h] = t;
        }
        gptr[g + 1] = (int)gsrc.size();
    }
    CK(cudaMalloc(&M.ptr, gptr.size() * sizeof(int)));
    CK(cudaMalloc(&M.src, std::max<size_t>(gsrc.size(), 1) * sizeof(int)));
    CK(cudaMalloc(&M.tid, std::max<size_t>(gtid.size(), 4) * sizeof(int)));
    CK(cudaMemcpy(M.ptr, gptr.data(), gptr.size() * sizeof(int), cudaMemcpyHostToDevice));
    if (!gsrc.empty()) {
        CK(cudaMemcpy(M.src, gsrc.data(), gsrc.size() * sizeof(int), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(M.tid, gtid.data(), gtid.size() * sizeof(int), cudaMemcpyHostToDevice));
    }
    return MLF_OK;
}

int mixed_setup(Ctx* c) {
    if (c->m32.ready) return MLF_OK;
    const int nl = c->nlev;
    int st;
    if ((st = conv32(c, &c->m32.R, c->dR, (size_t)c->N * 2 * c->lv[nl].K))) return st;
    for (int n = 3; n <= nl; ++n) {
        Level& L = c->lv[n];
        Mixed32::Lv& M = c->m32.lv[n];
        if ((st = conv32(c, &M.T, L.dT, (size_t)L.ntrans * L.K))) return st;
        if ((st = up32(c, &M.wq, L.wq))) return st;
        if ((st = group_lists(c, L, 2, M.grp[0]))) return st;
        if ((st = group_lists(c, L, 4, M.grp[1]))) return st;
        if (n < nl) {
            if ((st = up32(c, &M.wth, L.wth))) return st;
            if ((st = up32(c, &M.wph, L.wph))) return st;
            if ((st = up32(c, &M.thT_w, L.thT_w))) return st;
            if ((st = up32(c, &M.phT_w, L.phT_w))) return st;
            std::vector<double2> sh(8 * (size_t)L.K);
            CK(cudaMemcpy(sh.data(), L.dshift, sh.size() * sizeof(double2), cudaMemcpyDeviceToHost));
            std::vector<float2> s32(sh.size());
            for (size_t i = 0; i < sh.size(); ++i) s32[i] = make_float2((float)sh[i].x, (float)sh[i].y);
            CK(cudaMalloc(&M.shift, s32.size() * sizeof(float2)));
            CK(cudaMemcpy(M.shift, s32.data(), s32.size() * sizeof(float2), cudaMemcpyHostToDevice));
        }
    }
    size_t mx2 = 0, mx3 = 0;
    for (int n = 3; n < nl; ++n) {
        mx2 = std::max(mx2, ((size_t)c->lv[n].K + (size_t)c->lv[n].L * 2 * c->lv[n + 1].L) * sizeof(float2));
        mx3 = std::max(mx3, (size_t)SEP_SLAB * 2 * (c->lv[n + 1].L + c->lv[n].L) * sizeof(float2));
    }
    int optin = 0;
    CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->dev));
    if (mx2 > (size_t)optin || mx3 > (size_t)optin) {
        c->err = "parent sampling grid too large for the shared-memory interpolation stages";
        return MLF_E_ARG;
    }
    // kernel-wide limit shared by all contexts: the device maximum (see configure_kernels)
    CK(cudaFuncSetAttribute(k_anterp_sep<float2, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    CK(cudaFuncSetAttribute(k_interp_sep<float2, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    CK(cudaStreamSynchronize(c->stream));
    c->m32.ready = 1;
    return MLF_OK;
}

static int ensure_fields32(Ctx* c, int nrhs) {
    if (c->m32.fcap >= nrhs && c->m32.xf) return MLF_OK;
    for (int n = 3; n <= c->nlev; ++n) {
        Mixed32::Lv& M = c->m32.lv[n];
        if (M.C) cudaFree(M.C);
        if (M.B) cudaFree(M.B);
        if (M.A) cudaFree(M.A);
        const size_t f = (size_t)c->lv[n].nb * nrhs * 2 * c->lv[n].K;
        CK(cudaMalloc(&M.C, f * sizeof(float2)));
        CK(cudaMalloc(&M.B, f * sizeof(float2)));
        CK(cudaMalloc(&M.A, f * sizeof(float2)));
    }
    if (c->m32.xf) cudaFree(c->m32.xf);
    CK(cudaMalloc(&c->m32.xf, (size_t)c->N * nrhs * sizeof(float2)));
    if (c->m32.xT) cudaFree(c->m32.xT);
    CK(cudaMalloc(&c->m32.xT, (size_t)c->N * nrhs * sizeof(float2)));
    c->m32.fcap = nrhs;
    return MLF_OK;
}

static int matvec32_core(Ctx* c, const double2* x, const float2* x32, double2* y, int nrhs, int ld, cudaStream_t s);

int device_matvec32(Ctx* c, const double2* x, double2* y, int nrhs, int ld, cudaStream_t s) {
    return matvec32_core(c, x, nullptr, y, nrhs, ld, s);
}

// y (FP64 columns, ld = N) = A32 x32 (FP32 packed columns)
int device_matvec32_from32(Ctx* c, const float2* x32, double2* y, int nrhs, cudaStream_t s) {
    return matvec32_core(c, nullptr, x32, y, nrhs, c->N, s);
}

// Field slots (columns x polarisations) per CTA of the separable passes: the
// largest of 8, 4, 2 that divides 2 nrhs and keeps the CTA within 48 KB of
// shared memory (four CTAs per SM), else 1.  The slots share every index and
// weight load of the stencils.
template <class F>
static void slots_dispatch(int nrhs, size_t per_slot, F f) {
    const size_t cap = 48 * 1024;
    if ((2 * nrhs) % 8 == 0 && 8 * per_slot <= cap) f(std::integral_constant<int, 8>());
    else if ((2 * nrhs) % 4 == 0 && 4 * per_slot <= cap) f(std::integral_constant<int, 4>());
    else if (2 * per_slot <= cap) f(std::integral_constant<int, 2>());
    else f(std::integral_constant<int, 1>());
}

static int matvec32_core(Ctx* c, const double2* x, const float2* x32, double2* y, int nrhs, int ld, cudaStream_t s) {
    int st;
    if (need_tree(c)) return MLF_E_STATE;
    if ((st = mixed_setup(c))) return st;
    if ((st = ensure_fields32(c, nrhs))) return st;
    const int nl = c->nlev;
    Level& leaf = c->lv[nl];
    const bool prof = c->profiling != 0;
    if (prof) cudaEventRecord(c->ev[0], s);
    const float2* xf = x32 ? x32 : c->m32.xf;
    if (nrhs == 1) {
        if (!x32) k32_pack_x<<<dim3((c->N + 255) / 256, nrhs), 256, 0, s>>>(c->N, nrhs, ld, x, c->m32.xf);
        k32_aggregate<<<leaf.nb * nrhs, 256, 0, s>>>(leaf.K, nrhs, c->N, c->dbox_ptr, c->dperm, c->m32.R, xf,
                                                     c->m32.lv[nl].C);
    } else {
        // blocks of columns: box-sorted row-major copy, then per-box GEMMs
        // (or one warp per basis for small boxes)
        if ((st = device_blk_pack(c, x, x32, ld, nrhs, c->m32.xT, s))) return st;
        const int eng = blk_engine_of(c);
        st = warp_engine(eng) ? device_agg_warp32(c, c->m32.R, leaf.K, c->m32.xT, nrhs, c->m32.lv[nl].C, s)
             : eng == 4       ? device_agg_tc(c, c->m32.R, leaf.K, c->m32.xT, nrhs, c->m32.lv[nl].C, s)
                              : device_agg_blocks32(c, c->m32.R, leaf.K, c->m32.xT, nrhs, c->m32.lv[nl].C, s);
        if (st) return st;
    }
    if (prof) cudaEventRecord(c->ev[1], s);
    for (int n = nl; n >= 4; --n) {
        Level& Lc = c->lv[n];
        Level& Lp = c->lv[n - 1];
        const int nslab = (Lp.L + SEP_SLAB - 1) / SEP_SLAB;
        const size_t per = (size_t)SEP_SLAB * 2 * (Lc.L + Lp.L) * sizeof(float2);   // child rows + parent slab
        const Mixed32::Lv &mp = c->m32.lv[n - 1], &mc = c->m32.lv[n];
        slots_dispatch(nrhs, per, [&](auto ns) {
            constexpr int NS = decltype(ns)::value;
            k_interp_sep<float2, NS><<<Lp.nb * (2 * nrhs / NS) * nslab, 256, NS * per, s>>>(
                Lp.L, Lc.L, nrhs, nslab, Lp.dchild_ptr, Lc.doctant, Lp.dsth, mp.wth, Lp.dsph, mp.wph, mp.shift, mc.C,
                mp.C);
        });
    }
    if (prof) cudaEventRecord(c->ev[2], s);
    for (int n = 3; n <= nl; ++n) {
        Level& L = c->lv[n];
        const int bd = 128, nch = (L.K + bd - 1) / bd;
        const int nr = nrhs <= 1 ? 1 : nrhs <= 2 ? 2 : nrhs <= 4 ? 4 : 8;
        const dim3 grid(L.nb * nch, (nrhs + nr - 1) / nr);
        const Mixed32::Lv& m = c->m32.lv[n];
        const int G = c->tr_group ? c->tr_group : (nrhs == 1 ? 2 : 4);
        if (G > 1 && m.grp[G / 4].ptr) {
            // box groups: at most 8 sums of each box's two polarisations per thread
            const Mixed32::Lv::Grp& gl = m.grp[G / 4];
            const int nrg = std::min(nr, c->tr_cols ? c->tr_cols : (G == 4 ? 2 : 4));
            const int ng = (L.nb + G - 1) / G;
            const dim3 gg(ng * nch, (nrhs + nrg - 1) / nrg);
#define TGRP(NR_, G_) k32_translate_grp<NR_, G_><<<gg, bd, 0, s>>>(L.K, L.nb, nrhs, nch, gl.ptr, gl.src, gl.tid, \
                                                                  m.T, m.wq, m.C, m.B)
            if (G == 4) {
                if (nrg == 1) TGRP(1, 4); else if (nrg == 2) TGRP(2, 4); else TGRP(4, 4);
            } else {
                if (nrg == 1) TGRP(1, 2); else if (nrg == 2) TGRP(2, 2); else TGRP(4, 2);
            }
#undef TGRP
            continue;
        }
        if (nr == 1)
            k32_translate<1><<<grid, bd, 0, s>>>(L.K, nrhs, nch, L.dfar_ptr, L.dfar_src, L.dfar_tid, m.T, m.wq, m.C, m.B);
        else if (nr == 2)
            k32_translate<2><<<grid, bd, 0, s>>>(L.K, nrhs, nch, L.dfar_ptr, L.dfar_src, L.dfar_tid, m.T, m.wq, m.C, m.B);
        else if (nr == 4)
            k32_translate<4><<<grid, bd, 0, s>>>(L.K, nrhs, nch, L.dfar_ptr, L.dfar_src, L.dfar_tid, m.T, m.wq, m.C, m.B);
        else
            k32_translate<8><<<grid, bd, 0, s>>>(L.K, nrhs, nch, L.dfar_ptr, L.dfar_src, L.dfar_tid, m.T, m.wq, m.C, m.B);
    }
    if (prof) cudaEventRecord(c->ev[3], s);
    for (int n = 4; n <= nl; ++n) {
        Level& Lc = c->lv[n];
        Level& Lp = c->lv[n - 1];
        const float2* Psrc = (n == 4) ? c->m32.lv[n - 1].B : c->m32.lv[n - 1].A;
        const size_t per = ((size_t)Lp.K + (size_t)Lp.L * 2 * Lc.L) * sizeof(float2);
        const Mixed32::Lv &mp = c->m32.lv[n - 1], &mc = c->m32.lv[n];
        slots_dispatch(nrhs, per, [&](auto ns) {
            constexpr int NS = decltype(ns)::value;
            k_anterp_sep<float2, NS><<<Lc.nb * (2 * nrhs / NS), 256, NS * per, s>>>(
                Lp.L, Lc.L, nrhs, Lc.dparent, Lc.doctant, Lp.dthT_ptr, Lp.dthT_row, mp.thT_w, Lp.dphT_ptr,
                Lp.dphT_row, mp.phT_w, mp.shift, Psrc, mc.B, mc.A);
        });
    }
    if (prof) cudaEventRecord(c->ev[4], s);
    {
        const long long warps = (long long)c->N * nrhs;
        const float facy = (float)(c->ph.w * MU / (4. * PI));
        if (nrhs == 1) {
            k32_receive_near<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, s>>>(
                leaf.K, c->N, nrhs, ld, c->dperm, c->dbox_of_sorted, c->m32.R, (nl == 3 ? c->m32.lv[nl].B : c->m32.lv[nl].A), c->dia, c->dja,
                c->dZ, xf, facy, y);
        } else if (warp_engine(blk_engine_of(c))) {
            if ((st = device_recv_near_warp32(c, c->m32.R, leaf.K, (nl == 3 ? c->m32.lv[nl].B : c->m32.lv[nl].A), facy,
                                              c->m32.xT, nrhs, ld, y, s)))
                return st;
        } else {
            const float2* Aleaf = nl == 3 ? c->m32.lv[nl].B : c->m32.lv[nl].A;
            if (blk_engine_of(c) == 4) {
                // the X operand was packed by the aggregation of this product
                if ((st = device_recv_tc(c, c->m32.R, leaf.K, Aleaf, facy, nrhs, ld, y, s))) return st;
                st = device_near_tc(c, c->m32.xT, ld, nrhs, y, s, true);
            } else {
                if ((st = device_recv_blocks32(c, c->m32.R, leaf.K, Aleaf, facy, nrhs, ld, y, s))) return st;
                st = device_near_blocks32(c, c->m32.xT, ld, nrhs, y, s);
            }
            if (st) return st;
        }
    }
    if (prof) cudaEventRecord(c->ev[5], s);
    if (!cuda_ok(c, cudaGetLastError(), "matvec32")) return MLF_E_CUDA;
    if (prof) {
        CK(cudaEventSynchronize(c->ev[5]));
        for (int i = 0; i < 5; ++i) cudaEventElapsedTime(&c->stage_ms[i], c->ev[i], c->ev[i + 1]);
    }
    return MLF_OK;
}

void mixed_free(Ctx* c) {
    auto F = [](void* p) { if (p) cudaFree(p); };
    F(c->m32.R); F(c->m32.xf); F(c->m32.xT); F(c->mix_ws);
    c->mix_ws = nullptr;
    c->mix_ws_bytes = 0;
    for (int n = 0; n < 32; ++n) {
        Mixed32::Lv& M = c->m32.lv[n];
        F(M.T); F(M.wq); F(M.shift); F(M.C); F(M.B); F(M.A);
        F(M.wth); F(M.wph); F(M.thT_w); F(M.phT_w);
        for (auto& g : M.grp) { F(g.ptr); F(g.src); F(g.tid); }
    }
}

// ---------------------------------------------------------------------------
// GMRES-IR: FP64 iterative refinement, each step one right-preconditioned
// GMRES(m) cycle on the FP32 operator (classical Gram-Schmidt, one pass by
// default, two with mlf_set_gs_passes).
// The reference's CGS (kept as mode 0) is too erratic to tolerate an
// operator perturbed at the 1e-7 level; GMRES minimises the residual over
// the Krylov space and cannot diverge.
// ---------------------------------------------------------------------------

constexpr int GM_BLOCKS = 128;

__global__ void k_resid(size_t n, const double2* __restrict__ b, const double2* __restrict__ Ax,
                        double2* __restrict__ r) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        r[i] = make_double2(b[i].x - Ax[i].x, b[i].y - Ax[i].y);
}
__global__ void k_axpy1(size_t n, const double2* __restrict__ d, double2* __restrict__ x) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        x[i].x += d[i].x;
        x[i].y += d[i].y;
    }
}

// partial[(i*nrhs + col)*GM_BLOCKS + blk] = sum conj(V_i) w   (grid: GM_BLOCKS, nrhs, nvec)
// or, with V == nullptr, sum |w|^2 in the real part (nvec = 1).
__global__ void k_mdot(int N, int nrhs, const double2* __restrict__ V, size_t vstride, const double2* __restrict__ w,
                       double2* __restrict__ partial) {
    const int col = blockIdx.y, i = blockIdx.z;
    const double2* wc = w + (size_t)col * N;
    const double2* vc = V ? V + i * vstride + (size_t)col * N : nullptr;
    double sr = 0, si = 0;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < N; e += gridDim.x * blockDim.x) {
        const double2 b = wc[e];
        if (vc) {
            const double2 a = vc[e];   // conj(a) * b
            sr = fma(a.x, b.x, sr); sr = fma(a.y, b.y, sr);
            si = fma(a.x, b.y, si); si = fma(-a.y, b.x, si);
        } else {
            sr = fma(b.x, b.x, sr); sr = fma(b.y, b.y, sr);
        }
    }
    __shared__ double rs[256], is[256];
    rs[threadIdx.x] = sr;
    is[threadIdx.x] = si;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) { rs[threadIdx.x] += rs[threadIdx.x + s]; is[threadIdx.x] += is[threadIdx.x + s]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[((size_t)i * nrhs + col) * gridDim.x + blockIdx.x] = make_double2(rs[0], is[0]);
}

// out[k] = sum_b partial[k*GM_BLOCKS + b], fixed order
__global__ void k_reduce_partials(int nk, const double2* __restrict__ partial, double2* __restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nk) return;
    double2 s = make_double2(0, 0);
    for (int b = 0; b < GM_BLOCKS; ++b) {
        s.x += partial[(size_t)k * GM_BLOCKS + b].x;
        s.y += partial[(size_t)k * GM_BLOCKS + b].y;
    }
    out[k] = s;
}

// FP32 Arnoldi kernels: basis V32 and work vector w32 in float, per-thread
// sums in float, block and final reductions in double.
__global__ void k_mdot32(int N, int nrhs, const float2* __restrict__ V, size_t vstride, const float2* __restrict__ w,
                         double2* __restrict__ partial) {
    const int col = blockIdx.y, i = blockIdx.z;
    const float2* wc = w + (size_t)col * N;
    const float2* vc = V ? V + i * vstride + (size_t)col * N : nullptr;
    float sr = 0.f, si = 0.f;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < N; e += gridDim.x * blockDim.x) {
        const float2 b = wc[e];
        if (vc) {
            const float2 a = vc[e];
            sr = fmaf(a.x, b.x, sr); sr = fmaf(a.y, b.y, sr);
            si = fmaf(a.x, b.y, si); si = fmaf(-a.y, b.x, si);
        } else {
            sr = fmaf(b.x, b.x, sr); sr = fmaf(b.y, b.y, sr);
        }
    }
    __shared__ double rs[256], is[256];
    rs[threadIdx.x] = sr;
    is[threadIdx.x] = si;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) { rs[threadIdx.x] += rs[threadIdx.x + s]; is[threadIdx.x] += is[threadIdx.x + s]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[((size_t)i * nrhs + col) * gridDim.x + blockIdx.x] = make_double2(rs[0], is[0]);
}

// Block dot products for the FP32 Arnoldi step: each CTA keeps its slice of
// w (MD_E values per thread) in registers and streams its share of the nvec
// basis vectors past it (blockIdx.z of gridDim.z shares, so that one column
// of 10^5 unknowns still fills the GPU), MD_G vectors per block reduction.
// partial[(i * nrhs + col) * gridDim.x + blockIdx.x] = sum conj(V_i) w over the slice.
constexpr int MD_E = 8, MD_G = 4;
template <class BT>
__global__ void __launch_bounds__(256) k_mdot32b(int N, int nrhs, int nvec, const BT* __restrict__ V,
                                                 size_t vstride, float ls, const float2* __restrict__ w,
                                                 double2* __restrict__ partial) {
    const int col = blockIdx.y;
    const size_t base = (size_t)col * N;
    const int e0 = blockIdx.x * 256 * MD_E + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ float red[8][2 * MD_G];
    float2 wv[MD_E];
#pragma unroll
    for (int u = 0; u < MD_E; ++u) {
        const int e = e0 + u * 256;
        wv[u] = e < N ? w[base + e] : make_float2(0.f, 0.f);
    }
    const int vper = ((nvec + gridDim.z - 1) / gridDim.z + MD_G - 1) / MD_G * MD_G;
    const int iend = min(nvec, (int)(blockIdx.z + 1) * vper);
    for (int i0 = blockIdx.z * vper; i0 < iend; i0 += MD_G) {
        float sacc[2 * MD_G];
#pragma unroll
        for (int g = 0; g < MD_G; ++g) {
            float sr = 0.f, si = 0.f;
            const int i = i0 + g;
            if (i < iend) {
                const BT* v = V + (size_t)i * vstride + base;
#pragma unroll
                for (int u = 0; u < MD_E; ++u) {
                    const int e = e0 + u * 256;
                    if (e < N) {
                        const float2 a = bload(v + e, ls);
                        sr = fmaf(a.x, wv[u].x, sr); sr = fmaf(a.y, wv[u].y, sr);
                        si = fmaf(a.x, wv[u].y, si); si = fmaf(-a.y, wv[u].x, si);
                    }
                }
            }
            sacc[2 * g] = sr;
            sacc[2 * g + 1] = si;
        }
        // warp sums of the 2 MD_G values by halving exchanges (MD_G = 4: 9
        // shuffles instead of 40): lane L ends with value (L >> 2)'s total
        static_assert(2 * MD_G == 8, "the exchange below is written for 8 values");
#pragma unroll
        for (int st = 0; st < 3; ++st) {
            const int o = 16 >> st, h = 4 >> st;
            const bool up = (lane & o) != 0;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (q < h) {
                    const float send = up ? sacc[q] : sacc[q + h];
                    const float keep = up ? sacc[q + h] : sacc[q];
                    sacc[q] = keep + __shfl_xor_sync(0xffffffffu, send, o);
                }
            }
        }
        sacc[0] += __shfl_xor_sync(0xffffffffu, sacc[0], 2);
        sacc[0] += __shfl_xor_sync(0xffffffffu, sacc[0], 1);
        if ((lane & 3) == 0) red[warp][lane >> 2] = sacc[0];
        __syncthreads();
        if (threadIdx.x < MD_G && i0 + (int)threadIdx.x < iend) {
            double tr = 0, ti = 0;
            for (int wp = 0; wp < 8; ++wp) {
                tr += red[wp][2 * threadIdx.x];
                ti += red[wp][2 * threadIdx.x + 1];
            }
            partial[((size_t)(i0 + threadIdx.x) * nrhs + col) * gridDim.x + blockIdx.x] = make_double2(tr, ti);
        }
        __syncthreads();
    }
}

// out[k] = sum_b partial[k * nb + b], fixed order
__global__ void k_reduce_partials_n(int nk, int nb, const double2* __restrict__ partial, double2* __restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nk) return;
    double2 s = make_double2(0, 0);
    for (int b = 0; b < nb; ++b) {
        s.x += partial[(size_t)k * nb + b].x;
        s.y += partial[(size_t)k * nb + b].y;
    }
    out[k] = s;
}

template <class BT>
__global__ void k_gs_update32(int N, int nrhs, int nvec, const BT* __restrict__ V, size_t vstride, float ls,
                              const double2* __restrict__ h, float2* __restrict__ w) {
    const int col = blockIdx.y;
    __shared__ float2 hs[2048];
    for (int i = threadIdx.x; i < nvec; i += blockDim.x) {
        const double2 hd = h[(size_t)i * nrhs + col];
        hs[i] = make_float2((float)hd.x, (float)hd.y);
    }
    __syncthreads();
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < N; e += gridDim.x * blockDim.x) {
        float2 acc = w[(size_t)col * N + e];
        const BT* v = V + (size_t)col * N + e;
#pragma unroll 4
        for (int i = 0; i < nvec; ++i) {
            const float2 hv = hs[i];
            const float2 a = bload(v + (size_t)i * vstride, ls);
            acc.x -= hv.x * a.x - hv.y * a.y;
            acc.y -= hv.x * a.y + hv.y * a.x;
        }
        w[(size_t)col * N + e] = acc;
    }
}

template <class BT>
__global__ void k_colscale_df(int N, const double2* __restrict__ src, const double* __restrict__ s,
                              BT* __restrict__ dst, float ss) {
    const int col = blockIdx.y;
    const double f = s[col];
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < N; e += gridDim.x * blockDim.x) {
        const double2 v = src[(size_t)col * N + e];
        bstore(dst + (size_t)col * N + e, make_float2((float)(v.x * f), (float)(v.y * f)), ss);
    }
}

template <class BT>
__global__ void k_colscale32(int N, const float2* __restrict__ src, const double* __restrict__ s,
                             BT* __restrict__ dst, float ss) {
    const int col = blockIdx.y;
    const float f = (float)s[col];
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < N; e += gridDim.x * blockDim.x) {
        const float2 v = src[(size_t)col * N + e];
        bstore(dst + (size_t)col * N + e, make_float2(v.x * f, v.y * f), ss);
    }
}

// FP32 copy of one basis block (the preconditioner's input)
template <class BT>
__global__ void k_basis32(size_t n, const BT* __restrict__ src, float ls, float2* __restrict__ dst) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = bload(src + i, ls);
}

// d[col] = sum_i y[i*nrhs+col] V32_i[col] in double (once per cycle)
template <class BT>
__global__ void k_combine32(int N, int nrhs, int nvec, const BT* __restrict__ V, size_t vstride, float ls,
                            const double2* __restrict__ y, double2* __restrict__ d) {
    const int col = blockIdx.y;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < N; e += gridDim.x * blockDim.x) {
        double2 acc = make_double2(0, 0);
        for (int i = 0; i < nvec; ++i) {
            const double2 yv = y[i * nrhs + col];
            const float2 v = bload(V + i * vstride + (size_t)col * N + e, ls);
            acc.x += yv.x * v.x - yv.y * v.y;
            acc.y += yv.x * v.y + yv.y * v.x;
        }
        d[(size_t)col * N + e] = acc;
    }
}

__global__ void k_d2f_m(size_t n, const double2* __restrict__ a, float2* __restrict__ b) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        b[i] = make_float2((float)a[i].x, (float)a[i].y);
}
__global__ void k_f2d_m(size_t n, const float2* __restrict__ a, double2* __restrict__ b) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        b[i] = make_double2((double)a[i].x, (double)a[i].y);
}

namespace {
struct Cx {
    double r, i;
};
inline Cx cx(double r, double i) { return {r, i}; }
inline Cx operator+(Cx a, Cx b) { return {a.r + b.r, a.i + b.i}; }
inline Cx operator-(Cx a, Cx b) { return {a.r - b.r, a.i - b.i}; }
inline Cx operator*(Cx a, Cx b) { return {a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r}; }
inline Cx conjx(Cx a) { return {a.r, -a.i}; }
inline double absx(Cx a) { return std::hypot(a.r, a.i); }
inline Cx divx(Cx a, Cx b) {
    const double d = b.r * b.r + b.i * b.i;
    return {(a.r * b.r + a.i * b.i) / d, (a.i * b.r - a.r * b.i) / d};
}
}  // namespace

static int col_norms(Ctx* c, int nrhs, const double2* w, double2* partial, double2* dred, std::vector<double2>& h,
                     std::vector<double>& out, cudaStream_t s) {
    k_mdot<<<dim3(GM_BLOCKS, nrhs, 1), 256, 0, s>>>(c->N, nrhs, nullptr, 0, w, partial);
    k_reduce_partials<<<(nrhs + 127) / 128, 128, 0, s>>>(nrhs, partial, dred);
    CK(cudaMemcpyAsync(h.data(), dred, nrhs * sizeof(double2), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    for (int col = 0; col < nrhs; ++col) out[col] = std::sqrt(h[col].x);
    return MLF_OK;
}

static int col_norms32(Ctx* c, int nrhs, const float2* w, double2* partial, double2* dred, std::vector<double2>& h,
                       std::vector<double>& out, cudaStream_t s) {
    k_mdot32<<<dim3(GM_BLOCKS, nrhs, 1), 256, 0, s>>>(c->N, nrhs, nullptr, 0, w, partial);
    k_reduce_partials<<<(nrhs + 127) / 128, 128, 0, s>>>(nrhs, partial, dred);
    CK(cudaMemcpyAsync(h.data(), dred, nrhs * sizeof(double2), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    for (int col = 0; col < nrhs; ++col) out[col] = std::sqrt(h[col].x);
    return MLF_OK;
}

// FP64 M^-1 applied to the correction once per cycle
static int apply_precond64(Ctx* c, int precond, int nrhs, const double2* in, double2* out, cudaStream_t s) {
    if (precond == 2) return device_nearinv_apply(c, in, out, nrhs, s);
    if (precond == 1) {
        for (int col = 0; col < nrhs; ++col) {
            const int st = device_ilu_solve(c, in + (size_t)col * c->N, out + (size_t)col * c->N, s);
            if (st) return st;
        }
        return MLF_OK;
    }
    CK(cudaMemcpyAsync(out, in, (size_t)c->N * nrhs * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    return MLF_OK;
}

// Iterative refinement: r = b - A64 x (FP64); one cycle of right-preconditioned
// GMRES(m) with an all-FP32 inner loop (basis, Gram-Schmidt, preconditioner,
// operator; Hessenberg and Givens on the host in double); d = V y in double;
// x += M^-1 d (the neighbourhood inverse in FP32 as in the cycle, ILU0 in FP64).
// BT: the Krylov basis storage, float2 or __half2 (mlf_set_basis_precision).
template <class BT>
static int solve_mixed_t(Ctx* c, const double2* b, const double2* x0, double tol, int maxit, int nrhs, double2* x,
                         int* iters, double* relres, int precond, int* status, double inner_tol, int* outer) {
    const int N = c->N;
    // restart length: the one set, else 1600 while the basis fits in 16 GB,
    // down to 800 for wide blocks (a cold solve of the bench workloads takes
    // 1200-1600 steps; warm-started ones 500-800)
    const size_t colbytes = (size_t)N * nrhs * sizeof(BT);
    const int m_auto = (int)std::max<size_t>(800, std::min<size_t>(1600, ((size_t)16 << 30) / colbytes - 1));
    const int m = std::max(4, std::min(c->gmres_m > 0 ? c->gmres_m : m_auto, 2000));
    const size_t V1 = (size_t)N * nrhs;
    cudaStream_t s = c->stream;
    constexpr bool f32 = std::is_same<BT, float2>::value;
    const float ss = f32 ? 1.f : (float)std::sqrt((double)N), ls = 1.f / ss;   // store / load scales
    BT* V = nullptr;
    float2 *w32 = nullptr, *t32 = nullptr;
    double2 *w = nullptr, *r = nullptr, *t64 = nullptr, *partial = nullptr, *dred = nullptr;
    double* dscale = nullptr;
    const int md_chunks = (N + 256 * MD_E - 1) / (256 * MD_E);
    int nsm = 0;
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->dev));
    // The buffers come from a workspace the context keeps between solves: a
    // batched sweep solves hundreds of blocks, and allocating and freeing the
    // Krylov basis (tens of GB for wide blocks) for each took about 0.1 s.
    {
        auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
        const size_t sz[9] = {(size_t)(m + 1) * V1 * sizeof(BT), V1 * sizeof(float2), V1 * sizeof(float2),
                              V1 * sizeof(double2), V1 * sizeof(double2), V1 * sizeof(double2),
                              (size_t)(m + 1) * nrhs * std::max(GM_BLOCKS, md_chunks) * sizeof(double2),
                              (size_t)(m + 1) * nrhs * sizeof(double2), nrhs * sizeof(double)};
        size_t total = 0;
        for (size_t b : sz) total += al(b);
        if (c->mix_ws_bytes < total) {
            if (c->mix_ws) cudaFree(c->mix_ws);
            c->mix_ws = nullptr;
            c->mix_ws_bytes = 0;
            CK(cudaMalloc(&c->mix_ws, total));
            c->mix_ws_bytes = total;
        }
        char* p = static_cast<char*>(c->mix_ws);
        auto take = [&](int k) {
            char* q = p;
            p += al(sz[k]);
            return static_cast<void*>(q);
        };
        V = static_cast<BT*>(take(0));
        w32 = static_cast<float2*>(take(1));
        t32 = static_cast<float2*>(take(2));
        w = static_cast<double2*>(take(3));
        r = static_cast<double2*>(take(4));
        t64 = static_cast<double2*>(take(5));
        partial = static_cast<double2*>(take(6));
        dred = static_cast<double2*>(take(7));
        dscale = static_cast<double*>(take(8));
    }
    if (x0) CK(cudaMemcpyAsync(x, x0, V1 * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    else CK(cudaMemsetAsync(x, 0, V1 * sizeof(double2), s));
    const unsigned g = (unsigned)std::min<size_t>((N + 255) / 256, 2048);
    const dim3 gc(g, nrhs);
    std::vector<double2> hbuf((size_t)(m + 1) * nrhs);
    std::vector<double> bn(nrhs), beta(nrhs), scl(nrhs);
    if (int st = col_norms(c, nrhs, b, partial, dred, hbuf, bn, s)) return st;
    std::fill(iters, iters + nrhs, 0);
    std::vector<int> done(nrhs, 0);
    // stagnation: the best FP64 residual of each column and the inner step count that reached it
    std::vector<double> sbest(nrhs, HUGE_VAL);
    std::vector<int> sbest_it(nrhs, 0);
    // H: per column the (m + 1) x m Hessenberg matrix, left uninitialised (for
    // wide blocks it spans hundreds of MB of which a cycle touches the first
    // few hundred columns): every entry is written before it is read
    std::unique_ptr<Cx[]> H(new Cx[(size_t)nrhs * (m + 1) * m]);
    std::vector<Cx> G((size_t)nrhs * (m + 1)), CS((size_t)nrhs * m), SN((size_t)nrhs * m);
    auto Hc = [&](int col, int i, int j) -> Cx& { return H[((size_t)col * m + j) * (m + 1) + i]; };
    int st = MLF_OK, k = 0;
    const int max_outer = 1000;
    const bool prof = c->profiling != 0;
    if (prof) {
        for (int q = 0; q < 4; ++q)
            if (!c->sev[q]) CK(cudaEventCreate(&c->sev[q]));
        for (double& v : c->solve_ms) v = 0;
    }
    const auto t_start = std::chrono::steady_clock::now();
    for (; k < max_outer; ++k) {
        // The residual that decides convergence is always FP64.  Two first
        // steps need no FP64 operator: with no initial guess r = b exactly;
        // with a warm start, the first cycle's right-hand side b - Z x0 is
        // formed with the FP32 operator and only feeds the inner solve (no
        // column is declared converged on it), the FP64 residual after the
        // cycle deciding as always.
        const bool provisional = k == 0 && x0 != nullptr;
        if (prof) cudaStreamSynchronize(s);
        const auto t_res = std::chrono::steady_clock::now();
        if (k == 0 && !x0) {
            CK(cudaMemcpyAsync(r, b, V1 * sizeof(double2), cudaMemcpyDeviceToDevice, s));
        } else {
            // after a check, only the columns still running need a new residual
            // (a converged column's x and r no longer change): they are gathered
            // so that the FP64 operator runs on those columns alone
            std::vector<int> run;
            if (!provisional)
                for (int col = 0; col < nrhs; ++col)
                    if (!done[col]) run.push_back(col);
            const int nrun = (int)run.size();
            c->mv_prec = provisional ? 1 : 0;
            if (!provisional && nrun < nrhs) {
                for (int i = 0; i < nrun && !st; ++i)
                    if (!cuda_ok(c, cudaMemcpyAsync(w + (size_t)i * N, x + (size_t)run[i] * N, N * sizeof(double2),
                                                    cudaMemcpyDeviceToDevice, s), "gather"))
                        st = MLF_E_CUDA;
                if (!st && nrun) st = device_matvec(c, w, t64, nrun, N, s);
                c->mv_prec = 0;
                if (st) break;
                for (int i = 0; i < nrun; ++i)
                    k_resid<<<1024, 256, 0, s>>>((size_t)N, b + (size_t)run[i] * N, t64 + (size_t)i * N,
                                                 r + (size_t)run[i] * N);
            } else {
                st = device_matvec(c, x, t64, nrhs, N, s);
                c->mv_prec = 0;
                if (st) break;
                k_resid<<<4096, 256, 0, s>>>(V1, b, t64, r);
            }
        }
        if ((st = col_norms(c, nrhs, r, partial, dred, hbuf, beta, s))) break;
        if (prof) {   // col_norms synchronised the stream
            const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_res).count();
            c->solve_ms[provisional ? 5 : 4] += ms;
        }
        bool all = true, budget = false;
        for (int col = 0; col < nrhs; ++col) {
            // a NaN or Inf in b or in the residual ends the column first
            // (bn > 0 is false for a NaN norm, which would read as converged)
            const bool finite = std::isfinite(bn[col]) && std::isfinite(beta[col]);
            relres[col] = !finite ? beta[col] / bn[col] : (bn[col] > 0 ? beta[col] / bn[col] : 0.0);
            if (!finite && !done[col]) { done[col] = 1; status[col] = MLF_CGS_NOT_FINITE; }
            if (!done[col] && !provisional && (relres[col] < tol || bn[col] == 0)) {
                done[col] = 1;
                status[col] = MLF_CGS_CONVERGED;
            }
            if (c->stag_window > 0 && !done[col] && !provisional) {
                if (relres[col] < sbest[col]) {
                    sbest[col] = relres[col];
                    sbest_it[col] = iters[col];
                } else if (iters[col] - sbest_it[col] >= c->stag_window) {
                    done[col] = 1;
                    status[col] = MLF_CGS_STAGNATED;
                }
            }
            all = all && done[col];
            budget = budget || (!done[col] && iters[col] < maxit);
        }
        if (all || !budget) break;
        for (int col = 0; col < nrhs; ++col) scl[col] = (!done[col] && beta[col] > 0) ? 1.0 / beta[col] : 0.0;
        CK(cudaMemcpyAsync(dscale, scl.data(), nrhs * sizeof(double), cudaMemcpyHostToDevice, s));
        k_colscale_df<BT><<<gc, 256, 0, s>>>(N, r, dscale, V, ss);
        std::fill(G.begin(), G.end(), cx(0, 0));
        for (int col = 0; col < nrhs; ++col) G[(size_t)col * (m + 1)] = cx(done[col] ? 0.0 : beta[col], 0);
        std::vector<int> jcol(nrhs, 0), live(nrhs, 0);
        for (int col = 0; col < nrhs; ++col) live[col] = !done[col];
        cudaGraphExec_t gexec = nullptr;
        for (int j = 0; j < m; ++j) {
            bool any = false;
            for (int col = 0; col < nrhs; ++col) any = any || live[col];
            if (!any) break;
            if (prof) cudaEventRecord(c->sev[0], s);
            const float2* vj;
            if (f32) {
                vj = reinterpret_cast<const float2*>(V + (size_t)j * V1);
            } else {   // w32 is free until the operator writes it below
                k_basis32<BT><<<4096, 256, 0, s>>>(V1, V + (size_t)j * V1, ls, w32);
                vj = w32;
            }
            if (precond == 2) {
                if ((st = device_nearinv_apply32(c, vj, t32, nrhs, s))) break;
            } else if (precond == 1) {
                k_f2d_m<<<4096, 256, 0, s>>>(V1, vj, w);
                if ((st = apply_precond64(c, 1, nrhs, w, t64, s))) break;
                k_d2f_m<<<4096, 256, 0, s>>>(V1, t64, t32);
            } else {
                CK(cudaMemcpyAsync(t32, vj, V1 * sizeof(float2), cudaMemcpyDeviceToDevice, s));
            }
            if (prof) cudaEventRecord(c->sev[1], s);
            // w32 = float(A32 t32): the first step of a cycle records these
            // launches (fixed buffers) into a CUDA graph, later steps replay it
            if (!gexec) {
                if ((st = device_matvec32_from32(c, t32, w, nrhs, s))) break;   // allocates lazily, uncaptured
                k_d2f_m<<<4096, 256, 0, s>>>(V1, w, w32);
                cudaGraph_t graph = nullptr;
                if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
                    const int prof = c->profiling;
                    c->profiling = 0;
                    const int st2 = device_matvec32_from32(c, t32, w, nrhs, s);
                    k_d2f_m<<<4096, 256, 0, s>>>(V1, w, w32);
                    c->profiling = prof;
                    if (cudaStreamEndCapture(s, &graph) == cudaSuccess && st2 == MLF_OK && graph) {
                        if (cudaGraphInstantiate(&gexec, graph, 0) != cudaSuccess) gexec = nullptr;
                    }
                    if (graph) cudaGraphDestroy(graph);
                    cudaGetLastError();
                }
            } else {
                CK(cudaGraphLaunch(gexec, s));
            }
            if (prof) cudaEventRecord(c->sev[2], s);
            std::vector<double2> hsum((size_t)(j + 1) * nrhs, make_double2(0, 0));
            for (int pass = 0; pass < c->gs_passes; ++pass) {
                // vector shares when the slices alone leave SMs idle (under two CTAs
                // per SM): about four CTAs per SM in all, at least MD_G vectors each
                const int base_ctas = md_chunks * nrhs;
                const int vz = base_ctas >= 2 * nsm ? 1
                                                    : std::max(1, std::min((j + 1 + MD_G - 1) / MD_G,
                                                                           (4 * nsm + base_ctas - 1) / base_ctas));
                k_mdot32b<BT><<<dim3(md_chunks, nrhs, vz), 256, 0, s>>>(N, nrhs, j + 1, V, V1, ls, w32, partial);
                k_reduce_partials_n<<<((j + 1) * nrhs + 127) / 128, 128, 0, s>>>((j + 1) * nrhs, md_chunks, partial,
                                                                                  dred);
                k_gs_update32<BT><<<gc, 256, 0, s>>>(N, nrhs, j + 1, V, V1, ls, dred, w32);
                CK(cudaMemcpyAsync(hbuf.data(), dred, (size_t)(j + 1) * nrhs * sizeof(double2), cudaMemcpyDeviceToHost, s));
                CK(cudaStreamSynchronize(s));
                for (size_t q = 0; q < (size_t)(j + 1) * nrhs; ++q) { hsum[q].x += hbuf[q].x; hsum[q].y += hbuf[q].y; }
            }
            std::vector<double> hn(nrhs);
            if ((st = col_norms32(c, nrhs, w32, partial, dred, hbuf, hn, s))) break;
            for (int col = 0; col < nrhs; ++col) scl[col] = (live[col] && hn[col] > 1e-300) ? 1.0 / hn[col] : 0.0;
            CK(cudaMemcpyAsync(dscale, scl.data(), nrhs * sizeof(double), cudaMemcpyHostToDevice, s));
            k_colscale32<BT><<<gc, 256, 0, s>>>(N, w32, dscale, V + (size_t)(j + 1) * V1, ss);
            if (prof) {
                cudaEventRecord(c->sev[3], s);
                cudaEventSynchronize(c->sev[3]);
                float a = 0, b2 = 0, d = 0;
                cudaEventElapsedTime(&a, c->sev[0], c->sev[1]);
                cudaEventElapsedTime(&b2, c->sev[1], c->sev[2]);
                cudaEventElapsedTime(&d, c->sev[2], c->sev[3]);
                c->solve_ms[0] += a; c->solve_ms[1] += b2; c->solve_ms[2] += d;
            }
            for (int col = 0; col < nrhs; ++col) {
                if (!live[col]) continue;
                for (int i = 0; i <= j; ++i) Hc(col, i, j) = cx(hsum[(size_t)i * nrhs + col].x, hsum[(size_t)i * nrhs + col].y);
                Hc(col, j + 1, j) = cx(hn[col], 0);
                for (int i = 0; i < j; ++i) {
                    const Cx a = Hc(col, i, j), bq = Hc(col, i + 1, j);
                    const Cx c_ = CS[(size_t)col * m + i], s_ = SN[(size_t)col * m + i];
                    Hc(col, i, j) = conjx(c_) * a + conjx(s_) * bq;
                    Hc(col, i + 1, j) = cx(0, 0) - s_ * a + c_ * bq;
                }
                const Cx a = Hc(col, j, j), bq = Hc(col, j + 1, j);
                const double nrm = std::hypot(absx(a), absx(bq));
                Cx c_ = cx(1, 0), s_ = cx(0, 0);
                if (nrm > 0) { c_ = divx(a, cx(nrm, 0)); s_ = divx(bq, cx(nrm, 0)); }
                CS[(size_t)col * m + j] = c_;
                SN[(size_t)col * m + j] = s_;
                Hc(col, j, j) = cx(nrm, 0);
                Hc(col, j + 1, j) = cx(0, 0);
                const Cx gj = G[(size_t)col * (m + 1) + j];
                G[(size_t)col * (m + 1) + j] = conjx(c_) * gj;
                G[(size_t)col * (m + 1) + j + 1] = cx(0, 0) - s_ * gj;
                jcol[col] = j + 1;
                iters[col] += 1;
                const double est = absx(G[(size_t)col * (m + 1) + j + 1]);
                if (est < inner_tol * bn[col] || hn[col] <= 1e-300 * bn[col] || iters[col] >= maxit) live[col] = 0;
            }
        }
        if (gexec) cudaGraphExecDestroy(gexec);
        if (st) break;
        std::vector<double2> y((size_t)(m + 1) * nrhs, make_double2(0, 0));
        int jmax = 0;
        for (int col = 0; col < nrhs; ++col) {
            const int jj = jcol[col];
            jmax = std::max(jmax, jj);
            std::vector<Cx> yy(jj);
            for (int i = jj - 1; i >= 0; --i) {
                Cx acc = G[(size_t)col * (m + 1) + i];
                for (int q = i + 1; q < jj; ++q) acc = acc - Hc(col, i, q) * yy[q];
                yy[i] = Hc(col, i, i).r != 0 || Hc(col, i, i).i != 0 ? divx(acc, Hc(col, i, i)) : cx(0, 0);
            }
            for (int i = 0; i < jj; ++i) y[(size_t)i * nrhs + col] = make_double2(yy[i].r, yy[i].i);
        }
        if (jmax == 0) break;
        CK(cudaMemcpyAsync(dred, y.data(), (size_t)jmax * nrhs * sizeof(double2), cudaMemcpyHostToDevice, s));
        k_combine32<BT><<<gc, 256, 0, s>>>(N, nrhs, jmax, V, V1, ls, dred, w);
        if (precond == 2 && f32) {
            // the correction through the FP32 neighbourhood inverse the cycle itself
            // used (the FP64 apply of a 64-column block costs ~0.12 s on GB300's
            // FP64 units; the FP32 one changes the correction by ~1e-6 relative,
            // and the FP64 residual still decides).  With the FP16 basis the FP64
            // apply stays: a 3-column solve on that basis then ran into its step
            // limit, which it meets with the FP64 apply.
            k_d2f_m<<<4096, 256, 0, s>>>(V1, w, w32);
            if ((st = device_nearinv_apply32(c, w32, t32, nrhs, s))) break;
            k_f2d_m<<<4096, 256, 0, s>>>(V1, t32, t64);
        } else if ((st = apply_precond64(c, precond, nrhs, w, t64, s))) {
            break;
        }
        k_axpy1<<<4096, 256, 0, s>>>(V1, t64, x);
        CK(cudaGetLastError());
    }
    c->mv_prec = 0;
    for (int col = 0; col < nrhs; ++col)
        if (!done[col]) status[col] = MLF_CGS_MAXIT;
    *outer = k;
    if (!st && blk_engine_of(c) == 4) st = tc_check(c);
    if (prof) {
        cudaStreamSynchronize(s);
        c->solve_ms[3] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
        c->solve_ms[6] = k;
    }
    return st;
}

int device_solve_mixed(Ctx* c, const double2* b, const double2* x0, double tol, int maxit, int nrhs, double2* x,
                       int* iters, double* relres, int precond, int* status, double inner_tol, int* outer) {
    if (c->basis_bits == 16)
        return solve_mixed_t<__half2>(c, b, x0, tol, maxit, nrhs, x, iters, relres, precond, status, inner_tol, outer);
    return solve_mixed_t<float2>(c, b, x0, tol, maxit, nrhs, x, iters, relres, precond, status, inner_tol, outer);
}

}  // namespace mlf

using namespace mlf;

extern "C" int mlf_solve_times(mlf_ctx* h, double* out4) {
    if (!h || !out4) return MLF_E_ARG;
    for (int q = 0; q < 4; ++q) out4[q] = h->c.solve_ms[q];
    return MLF_OK;
}

extern "C" int mlf_solve_phases(mlf_ctx* h, double* out, int n) {
    if (!h || !out || n < 0) return MLF_E_ARG;
    for (int q = 0; q < n && q < 7; ++q) out[q] = h->c.solve_ms[q];
    return MLF_OK;
}

int mlf_set_gmres_restart(mlf_ctx* h, int m) {
    if (!h || (m != 0 && (m < 4 || m > 2000))) return MLF_E_ARG;
    h->c.gmres_m = m;
    return MLF_OK;
}

int mlf_set_gs_passes(mlf_ctx* h, int passes) {
    if (!h || passes < 1 || passes > 2) return MLF_E_ARG;
    h->c.gs_passes = passes;
    return MLF_OK;
}

int mlf_set_translation_group(mlf_ctx* h, int boxes, int cols) {
    if (!h || (boxes != 0 && boxes != 1 && boxes != 2 && boxes != 4) || (cols != 0 && cols != 1 && cols != 2 && cols != 4))
        return MLF_E_ARG;
    h->c.tr_group = boxes;
    h->c.tr_cols = cols;
    return MLF_OK;
}

int mlf_set_basis_precision(mlf_ctx* h, int bits) {
    if (!h || (bits != 16 && bits != 32)) return MLF_E_ARG;
    h->c.basis_bits = bits;
    return MLF_OK;
}

extern "C" int mlf_matvec32_device(mlf_ctx* h, const void* x, void* y, int nrhs, int ld, void* stream) {
    if (!h || !x || !y || nrhs <= 0 || ld < h->c.N) return MLF_E_ARG;
    Ctx* c = &h->c;
    if (!cuda_ok(c, cudaSetDevice(c->dev), "cudaSetDevice")) return MLF_E_CUDA;
    return device_matvec32(c, (const double2*)x, (double2*)y, nrhs, ld, stream ? (cudaStream_t)stream : c->stream);
}
