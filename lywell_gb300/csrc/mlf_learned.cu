// Learned near-field preconditioner: targets, tokens and installation.
//
// Base: the exact neighbourhood inverse M1 (mlf_nearinv): for each leaf box,
// the rows of inv(Z[S1, S1]) of its own bases, S1 = the bases of the 27-box
// neighbourhood (the near list), on the near CSR pattern.  The rows of the
// inverse over the larger 2-ring neighbourhood S2 (boxes within two leaf
// cells in every axis, 125 boxes) restricted to the same pattern, M2, make a
// better preconditioner but cost (125/27)^3 ~ 100 times more to build.  The
// network learns the correction D = M2 - M1 from local quantities, so the
// installed preconditioner M = M1 + scale * net(tokens) keeps M1's pattern,
// apply cost and linearity.
//
// A token is one near-field entry (row m, column j).  With s_m = 1/sqrt(Z_mm)
// (principal root) the scaled quantities are Zh = s_m Z_mj s_j,
// M1h = M1_mj / (s_m s_j), Dh = D_mj / (s_m s_j); features (16):
//   Re Zh, Im Zh, Re M1h, Im M1h, |M1h|, [same leaf box], [m == j],
//   (r_j - r_m) / lambda (3), |r_j - r_m| / lambda,
//   leaf-cell distance of the two boxes (max norm, Euclidean),
//   n_own(box of m) / 100, near boxes of that box / 27, 1;
// target (2): Re, Im of Dh.  No counterpart in the reference.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <unordered_map>
#include <vector>

#include "mlf_internal.h"
#include "mlf_zmn.cuh"

namespace mlf {

#define CK(call)                                             \
    do {                                                     \
        if (!cuda_ok(c, (call), #call)) return MLF_E_CUDA;   \
    } while (0)

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ float2 cdivf(float2 a, float2 b) {
    const float d = b.x * b.x + b.y * b.y;
    return make_float2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
__device__ __forceinline__ float2 csqrt_inv(float2 z) {
    const float r = sqrtf(sqrtf(z.x * z.x + z.y * z.y));
    const float th = 0.5f * atan2f(z.y, z.x);
    float sn, cs;
    sincosf(th, &sn, &cs);
    return make_float2(cs / r, -sn / r);
}
__device__ __forceinline__ int find_sorted(const int* S, int n, int v) {
    int lo = 0, hi = n - 1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        if (S[mid] == v) return mid;
        if (S[mid] < v) lo = mid + 1; else hi = mid - 1;
    }
    return -1;
}

// dense Z (complex(4), row-major N x N) for the 2-ring blocks
__global__ void k_lp_dense(int N, const double* __restrict__ t_baric, const double* __restrict__ t_baric_sub,
                           const double* __restrict__ p_coord, const int* __restrict__ e_t, const int* __restrict__ e_po,
                           const double* __restrict__ e_long, double w, double w_smue, double c72,
                           float2* __restrict__ Zd) {
    const int m = blockIdx.x;
    for (int n = threadIdx.x; n < N; n += blockDim.x) {
        const double2 v = zmn_mom(m, n, t_baric, t_baric_sub, p_coord, e_t, e_po, e_long, w, w_smue, c72);
        Zd[(size_t)m * N + n] = make_float2((float)v.x, (float)v.y);
    }
}

// s_m = 1/sqrt(Z_mm) from the near CSR diagonal
__global__ void k_lp_scale(int N, const int* __restrict__ ia, const int* __restrict__ ja, const float2* __restrict__ Z,
                           float2* __restrict__ s) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= N) return;
    const int q = ia[m] + find_sorted(ja + ia[m], ia[m + 1] - ia[m], m);
    s[m] = csqrt_inv(Z[q]);
}

// one warp per row m
__global__ void k_lp_tokens(int N, const int* __restrict__ ia, const int* __restrict__ ja,
                            const float2* __restrict__ Z, const double2* __restrict__ M1,
                            const float2* __restrict__ M2, const float2* __restrict__ s,
                            const int* __restrict__ box_of, const int* __restrict__ cell,
                            const int* __restrict__ nown, const int* __restrict__ nnear,
                            const double* __restrict__ e_centro, float inv_lambda, float* __restrict__ X,
                            float* __restrict__ T) {
    const int m = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (m >= N) return;
    const int bm = box_of[m];
    const float2 sm = s[m];
    for (int q = ia[m] + lane; q < ia[m + 1]; q += 32) {
        const int j = ja[q], bj = box_of[j];
        const float2 ss = cmulf(sm, s[j]);
        const float2 zh = cmulf(ss, Z[q]);
        const float2 m1 = make_float2((float)M1[q].x, (float)M1[q].y);
        const float2 m1h = cdivf(m1, ss);
        const float dx = (float)(e_centro[3 * j] - e_centro[3 * m]) * inv_lambda;
        const float dy = (float)(e_centro[3 * j + 1] - e_centro[3 * m + 1]) * inv_lambda;
        const float dz = (float)(e_centro[3 * j + 2] - e_centro[3 * m + 2]) * inv_lambda;
        const int cx = cell[3 * bj] - cell[3 * bm], cy = cell[3 * bj + 1] - cell[3 * bm + 1],
                  cz = cell[3 * bj + 2] - cell[3 * bm + 2];
        float* f = X + (size_t)q * 16;
        f[0] = zh.x;
        f[1] = zh.y;
        f[2] = m1h.x;
        f[3] = m1h.y;
        f[4] = sqrtf(m1h.x * m1h.x + m1h.y * m1h.y);
        f[5] = bm == bj ? 1.f : 0.f;
        f[6] = m == j ? 1.f : 0.f;
        f[7] = dx;
        f[8] = dy;
        f[9] = dz;
        f[10] = sqrtf(dx * dx + dy * dy + dz * dz);
        f[11] = (float)max(abs(cx), max(abs(cy), abs(cz)));
        f[12] = sqrtf((float)(cx * cx + cy * cy + cz * cz));
        f[13] = nown[bm] * 0.01f;
        f[14] = nnear[bm] * (1.f / 27.f);
        f[15] = 1.f;
        if (T) {
            const float2 d = make_float2(M2[q].x - m1.x, M2[q].y - m1.y);
            const float2 dh = cdivf(d, ss);
            T[2 * (size_t)q] = dh.x;
            T[2 * (size_t)q + 1] = dh.y;
        }
    }
}

// M = M1 + scale * s_m s_j (Y.x + j Y.y); counts non-finite outputs (set to zero)
__global__ void k_lp_install(int N, const int* __restrict__ ia, const int* __restrict__ ja,
                             const float2* __restrict__ s, const double2* __restrict__ M1,
                             const float* __restrict__ Y, float scale, double2* __restrict__ M,
                             int* __restrict__ nonfinite) {
    const int m = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (m >= N) return;
    const float2 sm = s[m];
    for (int q = ia[m] + lane; q < ia[m + 1]; q += 32) {
        float2 y = make_float2(Y[2 * (size_t)q], Y[2 * (size_t)q + 1]);
        if (!isfinite(y.x) || !isfinite(y.y)) {
            atomicAdd(nonfinite, 1);
            y = make_float2(0.f, 0.f);
        }
        const float2 d = cmulf(cmulf(sm, s[ja[q]]), y);
        M[q] = make_double2(M1[q].x + (double)(scale * d.x), M1[q].y + (double)(scale * d.y));
    }
}

// ---------------------------------------------------------------------------

struct LpHost {
    std::vector<int> cell, nown, nnear, box_of;
};

static int lp_host(Ctx* c, LpHost& H) {
    const int nl = c->nlev;
    const Level& leaf = c->lv[nl];
    const int nb = leaf.nb;
    double mn[3] = {1e300, 1e300, 1e300};
    for (int b = 0; b < nb; ++b)
        for (int d = 0; d < 3; ++d) mn[d] = std::min(mn[d], leaf.centre[3 * b + d]);
    H.cell.resize(3 * (size_t)nb);
    for (int b = 0; b < nb; ++b)
        for (int d = 0; d < 3; ++d) H.cell[3 * b + d] = (int)std::lround((leaf.centre[3 * b + d] - mn[d]) / leaf.side);
    H.nown.resize(nb);
    H.nnear.resize(nb);
    for (int b = 0; b < nb; ++b) {
        H.nown[b] = c->box_ptr[b + 1] - c->box_ptr[b];
        H.nnear[b] = c->nbox_ptr[b + 1] - c->nbox_ptr[b];
    }
    H.box_of = c->box_of;
    return MLF_OK;
}

struct LpDev {
    int *cell = nullptr, *nown = nullptr, *nnear = nullptr, *box_of = nullptr;
    float2* s = nullptr;
    void release() {
        for (void* p : {(void*)cell, (void*)nown, (void*)nnear, (void*)box_of, (void*)s})
            if (p) cudaFree(p);
        cell = nown = nnear = box_of = nullptr;
        s = nullptr;
    }
};

static int lp_upload(Ctx* c, const LpHost& H, LpDev& D) {
    auto up = [&](int** d, const std::vector<int>& v) -> bool {
        if (!cuda_ok(c, cudaMalloc(d, std::max<size_t>(v.size(), 1) * sizeof(int)), "alloc")) return false;
        return v.empty() || cuda_ok(c, cudaMemcpy(*d, v.data(), v.size() * sizeof(int), cudaMemcpyHostToDevice), "copy");
    };
    if (!up(&D.cell, H.cell) || !up(&D.nown, H.nown) || !up(&D.nnear, H.nnear) || !up(&D.box_of, H.box_of))
        return MLF_E_CUDA;
    CK(cudaMalloc(&D.s, (size_t)c->N * sizeof(float2)));
    k_lp_scale<<<(c->N + 255) / 256, 256, 0, c->stream>>>(c->N, c->dia, c->dja, c->dZ, D.s);
    CK(cudaGetLastError());
    return MLF_OK;
}

// M2 (near pattern, FP32) from the 2-ring inverses; bad: first singular box + 1
static int lp_ring_targets(Ctx* c, const LpHost& H, float2* M2, int* bad_box) {
    const int nl = c->nlev;
    const int nb = c->lv[nl].nb;
    const int N = c->N;
    if ((size_t)N * N * sizeof(float2) > ((size_t)24 << 30)) {
        c->err = "2-ring targets are generated on bodies up to 55 000 unknowns";
        return MLF_E_ARG;
    }
    // 2-ring lists: boxes within two cells (max norm), their bases sorted
    std::unordered_map<long long, int> at;
    auto key = [](int x, int y, int z) { return ((long long)(x + 4096) << 26) | ((long long)(y + 4096) << 13) | (z + 4096); };
    for (int b = 0; b < nb; ++b) at.emplace(key(H.cell[3 * b], H.cell[3 * b + 1], H.cell[3 * b + 2]), b);
    std::vector<long long> off(nb + 1, 0);
    std::vector<int> len(nb), bases;
    size_t ownmax = 0;
    for (int b = 0; b < nb; ++b) {
        const size_t start = bases.size();
        for (int dx = -2; dx <= 2; ++dx)
            for (int dy = -2; dy <= 2; ++dy)
                for (int dz = -2; dz <= 2; ++dz) {
                    auto it = at.find(key(H.cell[3 * b] + dx, H.cell[3 * b + 1] + dy, H.cell[3 * b + 2] + dz));
                    if (it == at.end()) continue;
                    const int j = it->second;
                    bases.insert(bases.end(), c->box_bases.begin() + c->box_ptr[j],
                                 c->box_bases.begin() + c->box_ptr[j + 1]);
                }
        std::sort(bases.begin() + start, bases.end());
        len[b] = (int)(bases.size() - start);
        off[b + 1] = (long long)bases.size();
        ownmax = std::max(ownmax, (size_t)(c->box_ptr[b + 1] - c->box_ptr[b]));
    }
    size_t fre = 0, tot = 0;
    CK(cudaMemGetInfo(&fre, &tot));
    const size_t zbytes = (size_t)N * N * sizeof(float2);
    if (zbytes + ((size_t)2 << 30) > fre) {
        c->err = "not enough device memory for the 2-ring targets";
        return MLF_E_NOMEM;
    }
    float2* Zd = nullptr;
    long long* doff = nullptr;
    int *dlen = nullptr, *dbases = nullptr;
    int st = MLF_OK;
    auto fail = [&](int code) { st = code; };
    if (!cuda_ok(c, cudaMalloc(&Zd, zbytes), "alloc") ||
        !cuda_ok(c, cudaMalloc(&doff, off.size() * sizeof(long long)), "alloc") ||
        !cuda_ok(c, cudaMalloc(&dlen, len.size() * sizeof(int)), "alloc") ||
        !cuda_ok(c, cudaMalloc(&dbases, std::max<size_t>(bases.size(), 1) * sizeof(int)), "alloc"))
        fail(MLF_E_CUDA);
    if (!st) {
        if (!cuda_ok(c, cudaMemcpy(doff, off.data(), off.size() * sizeof(long long), cudaMemcpyHostToDevice), "copy") ||
            !cuda_ok(c, cudaMemcpy(dlen, len.data(), len.size() * sizeof(int), cudaMemcpyHostToDevice), "copy") ||
            !cuda_ok(c, cudaMemcpy(dbases, bases.data(), bases.size() * sizeof(int), cudaMemcpyHostToDevice), "copy"))
            fail(MLF_E_CUDA);
    }
    if (!st) {
        const double c72 = (double)(1.0f / 72.0f);
        k_lp_dense<<<N, 256, 0, c->stream>>>(N, c->dt_baric, c->dt_baric_sub, c->dp_coord, c->de_t, c->de_po,
                                             c->de_long, c->ph.w, c->ph.w * c->ph.smue, c72, Zd);
        if (!cuda_ok(c, cudaGetLastError(), "dense Z")) fail(MLF_E_CUDA);
    }
    // blocked FP32 LU per box over its 2-ring list (mlf_nbhd_lu.cu)
    if (!st) st = ring_inverse_lu32(c, Zd, doff, dlen, dbases, len, off, (int)ownmax, M2, bad_box);
    for (void* p : {(void*)Zd, (void*)doff, (void*)dlen, (void*)dbases})
        if (p) cudaFree(p);
    return st;
}

int lp_tokens(Ctx* c, int with_target, float* X, float* T, long long cap, long long* ntok, int* bad_box) {
    if (need_tree(c)) return MLF_E_STATE;
    *ntok = c->nnz;
    if (bad_box) *bad_box = 0;
    if (!X) return MLF_OK;
    if (cap < c->nnz) {
        c->err = "token buffers too small";
        return MLF_E_ARG;
    }
    if (!(c->nearinv_ok && !c->nearinv_own)) {
        c->err = "tokens need the exact neighbourhood inverse (mlf_nearinv) first";
        return MLF_E_STATE;
    }
    const double2* M1 = c->dMinv_base ? c->dMinv_base : c->dMinv;
    LpHost H;
    int st;
    if ((st = lp_host(c, H))) return st;
    LpDev D;
    if ((st = lp_upload(c, H, D))) { D.release(); return st; }
    float2* M2 = nullptr;
    if (with_target) {
        if (!T) { D.release(); return MLF_E_ARG; }
        if (!cuda_ok(c, cudaMalloc(&M2, std::max<long long>(c->nnz, 1) * sizeof(float2)), "alloc")) {
            D.release();
            return MLF_E_CUDA;
        }
        int bad = 0;
        if ((st = lp_ring_targets(c, H, M2, &bad))) { cudaFree(M2); D.release(); return st; }
        if (bad_box) *bad_box = bad;
    }
    const long long threads = (long long)c->N * 32;
    k_lp_tokens<<<(unsigned)((threads + 255) / 256), 256, 0, c->stream>>>(
        c->N, c->dia, c->dja, c->dZ, M1, M2, D.s, D.box_of, D.cell, D.nown, D.nnear, c->de_centro,
        (float)(1.0 / c->ph.lambda), X, with_target ? T : nullptr);
    const bool okc = cuda_ok(c, cudaGetLastError(), "tokens") && cuda_ok(c, cudaStreamSynchronize(c->stream), "tokens");
    if (M2) cudaFree(M2);
    D.release();
    return okc ? MLF_OK : MLF_E_CUDA;
}

}  // namespace mlf

using namespace mlf;

extern "C" int mlf_lp_tokens(mlf_ctx* h, int with_target, float* X, float* T, long long cap, long long* ntok,
                             int* bad_box) {
    if (!h || !ntok) return MLF_E_ARG;
    Ctx* c = &h->c;
    if (!cuda_ok(c, cudaSetDevice(c->dev), "cudaSetDevice")) return MLF_E_CUDA;
    return lp_tokens(c, with_target, X, T, cap, ntok, bad_box);
}

extern "C" int mlf_mlp_forward(mlf_mlp* net, const float* X, long long ntok, float* Y, void* stream);

extern "C" int mlf_lp_install(mlf_ctx* h, mlf_mlp* net, float scale, int* nonfinite) {
    if (!h || !net || !nonfinite) return MLF_E_ARG;
    Ctx* c = &h->c;
    if (!cuda_ok(c, cudaSetDevice(c->dev), "cudaSetDevice")) return MLF_E_CUDA;
    if (need_tree(c)) return MLF_E_STATE;
    if (!(c->nearinv_ok && !c->nearinv_own)) {
        c->err = "mlf_lp_install needs the exact neighbourhood inverse (mlf_nearinv) first";
        return MLF_E_STATE;
    }
    const long long nnz = c->nnz;
    // keep the exact M1 so that installs can be repeated with other scales
    if (!c->dMinv_base) {
        CK(cudaMalloc(&c->dMinv_base, std::max<long long>(nnz, 1) * sizeof(double2)));
        CK(cudaMemcpy(c->dMinv_base, c->dMinv, nnz * sizeof(double2), cudaMemcpyDeviceToDevice));
    }
    float *X = nullptr, *Y = nullptr;
    int* dbad = nullptr;
    long long ntok = 0;
    int st = MLF_OK;
    if (!cuda_ok(c, cudaMalloc(&X, std::max<long long>(nnz, 1) * 16 * sizeof(float)), "alloc") ||
        !cuda_ok(c, cudaMalloc(&Y, std::max<long long>(nnz, 1) * 2 * sizeof(float)), "alloc") ||
        !cuda_ok(c, cudaMalloc(&dbad, sizeof(int)), "alloc") || !cuda_ok(c, cudaMemset(dbad, 0, sizeof(int)), "memset"))
        st = MLF_E_CUDA;
    if (!st) st = lp_tokens(c, 0, X, nullptr, nnz, &ntok, nullptr);
    if (!st && mlf_mlp_forward(net, X, ntok, Y, nullptr) != MLF_OK) {
        c->err = "network forward failed";
        st = MLF_E_CUDA;
    }
    LpHost H;
    LpDev D;
    if (!st) st = lp_host(c, H);
    if (!st) st = lp_upload(c, H, D);
    int hbad = 0;
    if (!st) {
        const long long threads = (long long)c->N * 32;
        k_lp_install<<<(unsigned)((threads + 255) / 256), 256, 0, c->stream>>>(c->N, c->dia, c->dja, D.s,
                                                                              c->dMinv_base, Y, scale, c->dMinv, dbad);
        if (!cuda_ok(c, cudaGetLastError(), "install") ||
            !cuda_ok(c, cudaMemcpyAsync(&hbad, dbad, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "install") ||
            !cuda_ok(c, cudaStreamSynchronize(c->stream), "install"))
            st = MLF_E_CUDA;
    }
    D.release();
    if (X) cudaFree(X);
    if (Y) cudaFree(Y);
    if (dbad) cudaFree(dbad);
    if (st) return st;
    if (c->dMinv32) { cudaFree(c->dMinv32); c->dMinv32 = nullptr; }   // FP32 copies rebuilt on next use
    if (c->dMinvblk) { cudaFree(c->dMinvblk); c->dMinvblk = nullptr; }
    tc_drop_precond(c);
    *nonfinite = hbad;
    c->learned = 1;
    return MLF_OK;
}
