// Learned near-field preconditioner: tokens, targets and installation.
//
// A token is one entry (p, q) of a leaf box's own near-field block Z_bb
// (llenarZesparcida's values, complex(4)), in the own-box compact order
// (box-major, row-major n_b x n_b blocks, offsets boff).  With the symmetric
// diagonal scaling s_p = 1 / sqrt(Z_pp) (principal root) and Zh = S Z S:
//   features (16): Re Zh_pq, Im Zh_pq, |Zh_pq|, [p == q],
//                  (r_q - r_p) / lambda (3), |r_q - r_p| / lambda,
//                  l_p / lambda, l_q / lambda, n_b / 100,
//                  sum_q' |Zh_pq'| / n_b, sum_p' |Zh_p'q| / n_b,
//                  Re, Im of Z_pp / |Z_pp|, 1
//   target  (2):   Re, Im of Mh_pq = M_pq / (s_p s_q) for an exact
//                  preconditioner M: the own-box inverse, or the rows of the
//                  leaf box's neighbourhood inverse restricted to its own
//                  columns.
// Installed, the network's outputs Mh give M_pq = s_p Mh_pq s_q in the
// own-box block storage, so the preconditioner is the same linear,
// block-diagonal apply as the own-box inverse.  No counterpart in the
// reference.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "mlf_internal.h"

namespace mlf {

#define CK(call)                                             \
    do {                                                     \
        if (!cuda_ok(c, (call), #call)) return MLF_E_CUDA;   \
    } while (0)

__device__ __forceinline__ float2 csqrt_inv(float2 z) {
    // 1 / sqrt(z), principal branch
    const float r = sqrtf(sqrtf(z.x * z.x + z.y * z.y));
    const float th = 0.5f * atan2f(z.y, z.x);
    float sn, cs;
    sincosf(th, &sn, &cs);
    return make_float2(cs / r, -sn / r);
}

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }

// own block of box b: column-major n_b x n_b at Zblk + self_off[b]
// s (per box-sorted position) = 1 / sqrt(Z_pp)
__global__ void k_lp_scale(int nb, const int* __restrict__ box_ptr, const long long* __restrict__ self_off,
                           const float2* __restrict__ Zblk, float2* __restrict__ s) {
    const int b = blockIdx.x;
    const int j0 = box_ptr[b], n = box_ptr[b + 1] - j0;
    const float2* Zs = Zblk + self_off[b];
    for (int p = threadIdx.x; p < n; p += blockDim.x) s[j0 + p] = csqrt_inv(Zs[(size_t)p * n + p]);
}

// features of every own-block entry of box b (one CTA per box)
__global__ void k_lp_features(const int* __restrict__ box_ptr, const long long* __restrict__ self_off,
                              const long long* __restrict__ tok_off, const float2* __restrict__ Zblk,
                              const float2* __restrict__ s, const int* __restrict__ perm,
                              const double* __restrict__ e_centro, const double* __restrict__ e_long, float inv_lambda,
                              float* __restrict__ X) {
    extern __shared__ float lp_sm[];
    const int b = blockIdx.x;
    const int j0 = box_ptr[b], n = box_ptr[b + 1] - j0;
    const float2* Zs = Zblk + self_off[b];
    float* rsum = lp_sm;
    float* csum = lp_sm + n;
    for (int p = threadIdx.x; p < n; p += blockDim.x) { rsum[p] = 0.f; csum[p] = 0.f; }
    __syncthreads();
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int p = e / n, q = e - p * n;
        const float2 zh = cmulf(cmulf(s[j0 + p], Zs[(size_t)q * n + p]), s[j0 + q]);
        const float a = sqrtf(zh.x * zh.x + zh.y * zh.y);
        atomicAdd(&rsum[p], a);
        atomicAdd(&csum[q], a);
    }
    __syncthreads();
    float* Xb = X + tok_off[b] * 16;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int p = e / n, q = e - p * n;
        const float2 zpq = Zs[(size_t)q * n + p];
        const float2 zh = cmulf(cmulf(s[j0 + p], zpq), s[j0 + q]);
        const int gp = perm[j0 + p], gq = perm[j0 + q];
        const float dx = (float)(e_centro[3 * gq] - e_centro[3 * gp]) * inv_lambda;
        const float dy = (float)(e_centro[3 * gq + 1] - e_centro[3 * gp + 1]) * inv_lambda;
        const float dz = (float)(e_centro[3 * gq + 2] - e_centro[3 * gp + 2]) * inv_lambda;
        const float2 zd = Zs[(size_t)p * n + p];
        const float zdn = sqrtf(zd.x * zd.x + zd.y * zd.y);
        float* f = Xb + (size_t)e * 16;
        f[0] = zh.x;
        f[1] = zh.y;
        f[2] = sqrtf(zh.x * zh.x + zh.y * zh.y);
        f[3] = p == q ? 1.f : 0.f;
        f[4] = dx;
        f[5] = dy;
        f[6] = dz;
        f[7] = sqrtf(dx * dx + dy * dy + dz * dz);
        f[8] = (float)e_long[gp] * inv_lambda;
        f[9] = (float)e_long[gq] * inv_lambda;
        f[10] = n * 0.01f;
        f[11] = rsum[p] / n;
        f[12] = csum[q] / n;
        f[13] = zd.x / zdn;
        f[14] = zd.y / zdn;
        f[15] = 1.f;
    }
}

// targets from the own-box inverse (compact row-major blocks at boff, FP64)
__global__ void k_lp_target_own(const int* __restrict__ box_ptr, const long long* __restrict__ boff,
                                const double2* __restrict__ M, const float2* __restrict__ s, float* __restrict__ T) {
    const int b = blockIdx.x;
    const int j0 = box_ptr[b], n = box_ptr[b + 1] - j0;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int p = e / n, q = e - p * n;
        const double2 m = M[boff[b] + e];
        const float2 sp = s[j0 + p], sq = s[j0 + q];
        const float2 ss = cmulf(sp, sq);
        const float den = ss.x * ss.x + ss.y * ss.y;
        // m / (s_p s_q)
        const float mx = (float)m.x, my = (float)m.y;
        T[(boff[b] + e) * 2] = (mx * ss.x + my * ss.y) / den;
        T[(boff[b] + e) * 2 + 1] = (my * ss.x - mx * ss.y) / den;
    }
}

// targets from the neighbourhood inverse (full CSR values in near order),
// restricted to the box's own columns
__global__ void k_lp_target_nbhd(const int* __restrict__ box_ptr, const long long* __restrict__ boff,
                                 const int* __restrict__ perm, const int* __restrict__ ia, const int* __restrict__ ja,
                                 const double2* __restrict__ M, const float2* __restrict__ s, float* __restrict__ T) {
    const int b = blockIdx.x;
    const int j0 = box_ptr[b], n = box_ptr[b + 1] - j0;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int p = e / n, q = e - p * n;
        const int m = perm[j0 + p], col = perm[j0 + q];
        int lo = ia[m], hi = ia[m + 1] - 1;
        double2 v = make_double2(0, 0);
        while (lo <= hi) {
            const int mid = (lo + hi) >> 1;
            if (ja[mid] == col) { v = M[mid]; break; }
            if (ja[mid] < col) lo = mid + 1; else hi = mid - 1;
        }
        const float2 ss = cmulf(s[j0 + p], s[j0 + q]);
        const float den = ss.x * ss.x + ss.y * ss.y;
        const float mx = (float)v.x, my = (float)v.y;
        T[(boff[b] + e) * 2] = (mx * ss.x + my * ss.y) / den;
        T[(boff[b] + e) * 2 + 1] = (my * ss.x - mx * ss.y) / den;
    }
}

// M_pq = s_p Mh_pq s_q into the own-box storage; counts non-finite outputs
__global__ void k_lp_install(const int* __restrict__ box_ptr, const long long* __restrict__ boff,
                             const float2* __restrict__ s, const float* __restrict__ Y, double2* __restrict__ M,
                             int* __restrict__ nonfinite) {
    const int b = blockIdx.x;
    const int j0 = box_ptr[b], n = box_ptr[b + 1] - j0;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int p = e / n, q = e - p * n;
        const long long t = boff[b] + e;
        float2 mh = make_float2(Y[2 * t], Y[2 * t + 1]);
        if (!isfinite(mh.x) || !isfinite(mh.y)) {
            atomicAdd(nonfinite, 1);
            mh = make_float2(0.f, 0.f);
        }
        const float2 v = cmulf(cmulf(s[j0 + p], mh), s[j0 + q]);
        M[t] = make_double2(v.x, v.y);
    }
}

struct LpLayout {
    std::vector<long long> boff, self_off;
    long long ntok = 0;
    int nmax = 0;
};

static int lp_layout(Ctx* c, LpLayout& L) {
    const int nb = (int)c->box_ptr.size() - 1;
    L.boff.assign(nb + 1, 0);
    L.self_off.assign(nb, -1);
    long long off = 0;
    for (int b = 0; b < nb; ++b) {
        const long long n = c->box_ptr[b + 1] - c->box_ptr[b];
        L.boff[b + 1] = L.boff[b] + n * n;
        L.nmax = std::max<int>(L.nmax, (int)n);
        for (int e = c->nbox_ptr[b]; e < c->nbox_ptr[b + 1]; ++e) {
            const int j = c->nbox_list[e];
            if (j == b) L.self_off[b] = off;
            off += n * (c->box_ptr[j + 1] - c->box_ptr[j]);
        }
        if (L.self_off[b] < 0) {
            c->err = "a leaf box is missing from its own near list";
            return MLF_E_STATE;
        }
    }
    L.ntok = L.boff[nb];
    return MLF_OK;
}

struct LpDev {
    long long* boff = nullptr;
    long long* self_off = nullptr;
    float2* s = nullptr;
};

static int lp_upload(Ctx* c, const LpLayout& L, LpDev& D) {
    const int nb = (int)c->box_ptr.size() - 1;
    CK(cudaMalloc(&D.boff, (nb + 1) * sizeof(long long)));
    CK(cudaMalloc(&D.self_off, nb * sizeof(long long)));
    CK(cudaMalloc(&D.s, (size_t)c->N * sizeof(float2)));
    CK(cudaMemcpy(D.boff, L.boff.data(), (nb + 1) * sizeof(long long), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(D.self_off, L.self_off.data(), nb * sizeof(long long), cudaMemcpyHostToDevice));
    k_lp_scale<<<nb, 128, 0, c->stream>>>(nb, c->dbox_ptr, D.self_off, c->dZblk, D.s);
    CK(cudaGetLastError());
    return MLF_OK;
}

static void lp_free(LpDev& D) {
    if (D.boff) cudaFree(D.boff);
    if (D.self_off) cudaFree(D.self_off);
    if (D.s) cudaFree(D.s);
}

int lp_tokens(Ctx* c, int target, float* X, float* T, long long cap, long long* ntok) {
    int st = near_blocks_ensure(c);
    if (st) return st;
    LpLayout L;
    if ((st = lp_layout(c, L))) return st;
    *ntok = L.ntok;
    if (!X) return MLF_OK;
    if (cap < L.ntok) {
        c->err = "token buffers too small";
        return MLF_E_ARG;
    }
    if (target == 1 && !(c->nearinv_ok && c->nearinv_own)) {
        c->err = "own-box targets need mlf_nearinv_own first";
        return MLF_E_STATE;
    }
    if (target == 2 && !(c->nearinv_ok && !c->nearinv_own)) {
        c->err = "neighbourhood targets need mlf_nearinv first";
        return MLF_E_STATE;
    }
    if (target && !T) return MLF_E_ARG;
    const int nb = (int)c->box_ptr.size() - 1;
    LpDev D;
    if ((st = lp_upload(c, L, D))) { lp_free(D); return st; }
    const size_t smem = 2 * (size_t)L.nmax * sizeof(float);
    if (smem > 48 * 1024) {
        lp_free(D);
        c->err = "leaf box too large for the feature kernel";
        return MLF_E_ARG;
    }
    k_lp_features<<<nb, 256, smem, c->stream>>>(c->dbox_ptr, D.self_off, D.boff, c->dZblk, D.s, c->dperm,
                                                c->de_centro, c->de_long, (float)(1.0 / c->ph.lambda), X);
    if (target == 1) k_lp_target_own<<<nb, 256, 0, c->stream>>>(c->dbox_ptr, c->dboff, c->dMinv, D.s, T);
    if (target == 2)
        k_lp_target_nbhd<<<nb, 256, 0, c->stream>>>(c->dbox_ptr, D.boff, c->dperm, c->dia, c->dja, c->dMinv, D.s, T);
    if (!cuda_ok(c, cudaGetLastError(), "tokens") || !cuda_ok(c, cudaStreamSynchronize(c->stream), "tokens")) {
        lp_free(D);
        return MLF_E_CUDA;
    }
    lp_free(D);
    return MLF_OK;
}

}  // namespace mlf

using namespace mlf;

extern "C" int mlf_lp_tokens(mlf_ctx* h, int target, float* X, float* T, long long cap, long long* ntok) {
    if (!h || !ntok || target < 0 || target > 2) return MLF_E_ARG;
    Ctx* c = &h->c;
    if (!cuda_ok(c, cudaSetDevice(c->dev), "cudaSetDevice")) return MLF_E_CUDA;
    return lp_tokens(c, target, X, T, cap, ntok);
}

extern "C" int mlf_mlp_forward(mlf_mlp* net, const float* X, long long ntok, float* Y, void* stream);

extern "C" int mlf_lp_install(mlf_ctx* h, mlf_mlp* net, int* nonfinite) {
    if (!h || !net || !nonfinite) return MLF_E_ARG;
    Ctx* c = &h->c;
    if (!cuda_ok(c, cudaSetDevice(c->dev), "cudaSetDevice")) return MLF_E_CUDA;
    long long ntok = 0;
    int st = lp_tokens(c, 0, nullptr, nullptr, 0, &ntok);
    if (st) return st;
    LpLayout L;
    if ((st = lp_layout(c, L))) return st;
    float *X = nullptr, *Y = nullptr;
    int* dbad = nullptr;
    CK(cudaMalloc(&X, std::max<long long>(ntok, 1) * 16 * sizeof(float)));
    CK(cudaMalloc(&Y, std::max<long long>(ntok, 1) * 2 * sizeof(float)));
    CK(cudaMalloc(&dbad, sizeof(int)));
    CK(cudaMemset(dbad, 0, sizeof(int)));
    if ((st = lp_tokens(c, 0, X, nullptr, ntok, &ntok))) { cudaFree(X); cudaFree(Y); cudaFree(dbad); return st; }
    if ((st = mlf_mlp_forward(net, X, ntok, Y, nullptr))) {
        c->err = "network forward failed";
        cudaFree(X); cudaFree(Y); cudaFree(dbad);
        return st;
    }
    // own-box storage, replacing any exact preconditioner
    if (c->dMinv) cudaFree(c->dMinv);
    if (c->dboff) cudaFree(c->dboff);
    if (c->dMinv32) cudaFree(c->dMinv32);
    c->dMinv = nullptr; c->dboff = nullptr; c->dMinv32 = nullptr;
    c->nearinv_ok = 0;
    const int nb = (int)c->box_ptr.size() - 1;
    LpDev D;
    if ((st = lp_upload(c, L, D))) { lp_free(D); cudaFree(X); cudaFree(Y); cudaFree(dbad); return st; }
    CK(cudaMalloc(&c->dMinv, std::max<long long>(ntok, 1) * sizeof(double2)));
    c->dboff = D.boff;
    D.boff = nullptr;
    c->minv_len = ntok;
    k_lp_install<<<nb, 256, 0, c->stream>>>(c->dbox_ptr, c->dboff, D.s, Y, c->dMinv, dbad);
    int hbad = 0;
    const bool okc = cuda_ok(c, cudaGetLastError(), "install") &&
                     cuda_ok(c, cudaMemcpyAsync(&hbad, dbad, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "install") &&
                     cuda_ok(c, cudaStreamSynchronize(c->stream), "install");
    lp_free(D);
    cudaFree(X); cudaFree(Y); cudaFree(dbad);
    if (!okc) return MLF_E_CUDA;
    *nonfinite = hbad;
    c->nearinv_own = 1;
    c->nearinv_ok = 1;
    c->learned = 1;
    return MLF_OK;
}
