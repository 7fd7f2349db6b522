// Separable interpolation / anterpolation between octree levels.
//
// The reference's stencil (llenarMinterp / hallarKcercanos / Wlagrange3,
// modMLFMA.f90:998-1341) gives each coarse sample (theta_i, phi_p) nine fine
// samples: three fine theta rows chosen by theta_i alone and three fine phi
// columns chosen by phi_p alone, weighted Wtheta(a) * Wphi(b).  It is a tensor
// product, so Interpolar (:1343-1365) is applied here as a theta pass then a
// phi pass, and Anterpolar (:1370-1390, its transpose) as the transposed phi
// pass then the transposed theta pass: 3 + 3 taps instead of 9 on the FP64
// pipe, with the same result up to rounding order.
//
// Field layout: F[((box * nrhs + r) * 2 + pol) * K + k], k = phi * L + theta.
#pragma once
#include <cuda_runtime.h>

#include "mlf_internal.h"   // SEP_SLAB

namespace mlf {

template <class V> struct CTraits;
template <> struct CTraits<double2> {
    typedef double R;
    static __device__ __forceinline__ double2 make(double a, double b) { return make_double2(a, b); }
};
template <> struct CTraits<float2> {
    typedef float R;
    static __device__ __forceinline__ float2 make(float a, float b) { return make_float2(a, b); }
};

// Upward pass for one parent box, one slab of coarse theta rows
// [i0, i0 + nr) and NS consecutive field slots (columns x polarisations of
// that box; NS divides 2 nrhs), which share every index and weight load.
// Y (smem, per slot [fine phi][row]) = theta pass of one child, threads along
// theta so the child field is read in contiguous runs; S (smem, per slot
// [coarse phi][row]) = the parent slab, summed over the children in box order
// (as the reference accumulates) and written once.
template <class V, int NS>
__global__ void k_interp_sep(int Lp, int Lc, int nrhs, int nslab, const int* __restrict__ child_ptr,
                             const int* __restrict__ octant, const int* __restrict__ sth,
                             const typename CTraits<V>::R* __restrict__ wth, const int* __restrict__ sph,
                             const typename CTraits<V>::R* __restrict__ wph, const V* __restrict__ shift,
                             const V* __restrict__ Cc, V* __restrict__ Cp) {
    typedef typename CTraits<V>::R R;
    constexpr int SL = SEP_SLAB;
    extern __shared__ __align__(16) unsigned char sep_smem[];
    const int s = blockIdx.x % nslab;
    const int pp0 = (blockIdx.x / nslab) * NS;   // first slot: (P * nrhs + r) * 2 + pol
    const int P = pp0 / (2 * nrhs);
    const int q0 = pp0 - P * 2 * nrhs;           // its place among the box's 2 nrhs slots
    const int i0 = s * SL;
    const int nr = min(SL, Lp - i0);
    const int Kp = Lp * 2 * Lp, Kc = Lc * 2 * Lc, Lc2 = 2 * Lc, Lp2 = 2 * Lp;
    V* Y = reinterpret_cast<V*>(sep_smem);        // NS x (2Lc x SL)
    V* S = Y + (size_t)NS * SL * Lc2;             // NS x (2Lp x SL)
    const int c0 = child_ptr[P], c1 = child_ptr[P + 1];
    for (int cb = c0; cb < c1; ++cb) {
        const V* src = Cc + ((size_t)cb * 2 * nrhs + q0) * Kc;   // slot u at src + u Kc
        for (int e = threadIdx.x; e < nr * Lc2; e += blockDim.x) {   // rows past nr are not visited
            const int jp = e / nr, li = e - jp * nr;
            const int it = i0 + li, ey = jp * SL + li;
            R w[3];
            int f[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) { w[a] = wth[3 * it + a]; f[a] = sth[3 * it + a] + jp * Lc; }
#pragma unroll
            for (int u = 0; u < NS; ++u) {
                const V* col = src + (size_t)u * Kc;
                R ax = 0, ay = 0;
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    const V v = col[f[a]];
                    ax = fma(w[a], v.x, ax);
                    ay = fma(w[a], v.y, ay);
                }
                Y[(size_t)u * SL * Lc2 + ey] = CTraits<V>::make(ax, ay);
            }
        }
        __syncthreads();
        const V* sh = shift + (size_t)octant[cb] * Kp;
        for (int e = threadIdx.x; e < nr * Lp2; e += blockDim.x) {
            const int ip = e / nr, li = e - ip * nr, es = ip * SL + li;
            const V z = sh[ip * Lp + i0 + li];
            R w[3];
            int f[3];
#pragma unroll
            for (int b = 0; b < 3; ++b) { w[b] = wph[3 * ip + b]; f[b] = sph[3 * ip + b] * SL + li; }
#pragma unroll
            for (int u = 0; u < NS; ++u) {
                const V* Yu = Y + (size_t)u * SL * Lc2;
                R vx = 0, vy = 0;
#pragma unroll
                for (int b = 0; b < 3; ++b) {
                    const V y = Yu[f[b]];
                    vx = fma(w[b], y.x, vx);
                    vy = fma(w[b], y.y, vy);
                }
                const R rx = vx * z.x - vy * z.y, ry = vx * z.y + vy * z.x;
                V* Su = S + (size_t)u * SL * Lp2;
                if (cb == c0) {
                    Su[es] = CTraits<V>::make(rx, ry);
                } else {
                    const V o = Su[es];
                    Su[es] = CTraits<V>::make(o.x + rx, o.y + ry);
                }
            }
        }
        __syncthreads();   // Y is refilled by the next child
    }
    for (int e = threadIdx.x; e < nr * Lp2; e += blockDim.x) {
        const int ip = e / nr, li = e - ip * nr, es = ip * SL + li;
#pragma unroll
        for (int u = 0; u < NS; ++u)
            Cp[(size_t)(pp0 + u) * Kp + ip * Lp + i0 + li] =
                c1 > c0 ? S[(size_t)u * SL * Lp2 + es] : CTraits<V>::make(0, 0);
    }
}

// Downward pass for one child box and NS consecutive field slots (columns x
// polarisations; NS divides 2 nrhs), which share every index and weight
// load: per slot D = parent * conj(shift) (smem, Kp), E = transposed phi pass
// (smem, Lp x 2Lc, stored [jp][it]), A = B + transposed theta pass.
template <class V, int NS>
__global__ void k_anterp_sep(int Lp, int Lc, int nrhs, const int* __restrict__ parent, const int* __restrict__ octant,
                             const int* __restrict__ thT_ptr, const int* __restrict__ thT_row,
                             const typename CTraits<V>::R* __restrict__ thT_w, const int* __restrict__ phT_ptr,
                             const int* __restrict__ phT_row, const typename CTraits<V>::R* __restrict__ phT_w,
                             const V* __restrict__ shift, const V* __restrict__ Psrc, const V* __restrict__ Bc,
                             V* __restrict__ Ac) {
    typedef typename CTraits<V>::R R;
    extern __shared__ __align__(16) unsigned char sep_smem[];
    const int Kp = Lp * 2 * Lp, Kc = Lc * 2 * Lc, Lc2 = 2 * Lc;
    V* D = reinterpret_cast<V*>(sep_smem);        // NS x Kp
    V* E = D + (size_t)NS * Kp;                   // NS x (Lp x 2Lc)
    const int slot0 = blockIdx.x * NS;            // (cb * nrhs + r) * 2 + pol
    const int cb = slot0 / (2 * nrhs), q0 = slot0 - cb * 2 * nrhs;
    const int P = parent[cb];
    const V* sh = shift + (size_t)octant[cb] * Kp;
    const V* src = Psrc + ((size_t)P * 2 * nrhs + q0) * Kp;   // slot u at src + u Kp
    for (int m = threadIdx.x; m < Kp; m += blockDim.x) {
        const V z = sh[m];
#pragma unroll
        for (int u = 0; u < NS; ++u) {
            const V v = src[(size_t)u * Kp + m];
            D[(size_t)u * Kp + m] = CTraits<V>::make(v.x * z.x + v.y * z.y, v.y * z.x - v.x * z.y);
        }
    }
    __syncthreads();
    const int nE = Lp * Lc2;
    for (int e = threadIdx.x; e < nE; e += blockDim.x) {
        const int jp = e / Lp, it = e - jp * Lp;
        R ax[NS], ay[NS];
#pragma unroll
        for (int u = 0; u < NS; ++u) ax[u] = ay[u] = 0;
        for (int q = phT_ptr[jp]; q < phT_ptr[jp + 1]; ++q) {
            const R w = phT_w[q];
            const int m = phT_row[q] * Lp + it;
#pragma unroll
            for (int u = 0; u < NS; ++u) {
                const V d = D[(size_t)u * Kp + m];
                ax[u] = fma(w, d.x, ax[u]);
                ay[u] = fma(w, d.y, ay[u]);
            }
        }
#pragma unroll
        for (int u = 0; u < NS; ++u) E[(size_t)u * nE + e] = CTraits<V>::make(ax[u], ay[u]);
    }
    __syncthreads();
    const size_t off = (size_t)slot0 * Kc;
    for (int e = threadIdx.x; e < Kc; e += blockDim.x) {
        const int jp = e / Lc, jt = e - jp * Lc;
        R ax[NS], ay[NS];
#pragma unroll
        for (int u = 0; u < NS; ++u) ax[u] = ay[u] = 0;
        for (int q = thT_ptr[jt]; q < thT_ptr[jt + 1]; ++q) {
            const R w = thT_w[q];
            const int m = jp * Lp + thT_row[q];
#pragma unroll
            for (int u = 0; u < NS; ++u) {
                const V v = E[(size_t)u * nE + m];
                ax[u] = fma(w, v.x, ax[u]);
                ay[u] = fma(w, v.y, ay[u]);
            }
        }
#pragma unroll
        for (int u = 0; u < NS; ++u) {
            const V bv = Bc[off + (size_t)u * Kc + e];
            Ac[off + (size_t)u * Kc + e] = CTraits<V>::make(bv.x + ax[u], bv.y + ay[u]);
        }
    }
}

}  // namespace mlf
