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

// Upward pass for one parent box, one column and polarisation, one slab of
// coarse theta rows [i0, i0 + nr).  Y (smem) = theta pass of one child:
// nr x 2Lc.  Children are added in box order, as the reference accumulates.
template <class V>
__global__ void k_interp_sep(int Lp, int Lc, int nrhs, int slab, int nslab, const int* __restrict__ child_ptr,
                             const int* __restrict__ octant, const int* __restrict__ sth,
                             const typename CTraits<V>::R* __restrict__ wth, const int* __restrict__ sph,
                             const typename CTraits<V>::R* __restrict__ wph, const V* __restrict__ shift,
                             const V* __restrict__ Cc, V* __restrict__ Cp) {
    typedef typename CTraits<V>::R R;
    extern __shared__ __align__(16) unsigned char sep_smem[];
    V* Y = reinterpret_cast<V*>(sep_smem);
    const int s = blockIdx.x % nslab;
    const int pp = blockIdx.x / nslab;          // (P * nrhs + r) * 2 + pol
    const int pol = pp & 1;
    const int Pr = pp >> 1;                     // P * nrhs + r
    const int P = Pr / nrhs, r = Pr % nrhs;
    const int i0 = s * slab;
    const int nr = min(slab, Lp - i0);
    const int Kp = Lp * 2 * Lp, Kc = Lc * 2 * Lc, Lc2 = 2 * Lc, Lp2 = 2 * Lp;
    V* out = Cp + (size_t)pp * Kp;
    const int c0 = child_ptr[P], c1 = child_ptr[P + 1];
    for (int cb = c0; cb < c1; ++cb) {
        const V* src = Cc + ((size_t)(cb * nrhs + r) * 2 + pol) * Kc;
        for (int e = threadIdx.x; e < nr * Lc2; e += blockDim.x) {
            const int li = e / Lc2, jp = e - li * Lc2;
            const int it = i0 + li;
            const V* col = src + (size_t)jp * Lc;
            R ax = 0, ay = 0;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const R w = wth[3 * it + a];
                const V v = col[sth[3 * it + a]];
                ax = fma(w, v.x, ax);
                ay = fma(w, v.y, ay);
            }
            Y[e] = CTraits<V>::make(ax, ay);
        }
        __syncthreads();
        const V* sh = shift + (size_t)octant[cb] * Kp;
        for (int e = threadIdx.x; e < nr * Lp2; e += blockDim.x) {
            const int ip = e / nr, li = e - ip * nr;
            const int k = ip * Lp + i0 + li;
            R vx = 0, vy = 0;
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                const R w = wph[3 * ip + b];
                const V y = Y[li * Lc2 + sph[3 * ip + b]];
                vx = fma(w, y.x, vx);
                vy = fma(w, y.y, vy);
            }
            const V z = sh[k];
            const R rx = vx * z.x - vy * z.y, ry = vx * z.y + vy * z.x;
            if (cb == c0) {
                out[k] = CTraits<V>::make(rx, ry);
            } else {
                const V o = out[k];
                out[k] = CTraits<V>::make(o.x + rx, o.y + ry);
            }
        }
        __syncthreads();
    }
}

// Downward pass for one child box, column and polarisation:
// D = parent * conj(shift) (smem, Kp), E = transposed phi pass (smem, Lp x 2Lc,
// stored [jp][it]), A = B + transposed theta pass.
template <class V>
__global__ void k_anterp_sep(int Lp, int Lc, int nrhs, const int* __restrict__ parent, const int* __restrict__ octant,
                             const int* __restrict__ thT_ptr, const int* __restrict__ thT_row,
                             const typename CTraits<V>::R* __restrict__ thT_w, const int* __restrict__ phT_ptr,
                             const int* __restrict__ phT_row, const typename CTraits<V>::R* __restrict__ phT_w,
                             const V* __restrict__ shift, const V* __restrict__ Psrc, const V* __restrict__ Bc,
                             V* __restrict__ Ac) {
    typedef typename CTraits<V>::R R;
    extern __shared__ __align__(16) unsigned char sep_smem[];
    const int Kp = Lp * 2 * Lp, Kc = Lc * 2 * Lc, Lc2 = 2 * Lc;
    V* D = reinterpret_cast<V*>(sep_smem);
    V* E = D + Kp;
    const int cr = blockIdx.x >> 1, pol = blockIdx.x & 1;   // cr = cb * nrhs + r
    const int cb = cr / nrhs, r = cr % nrhs;
    const int P = parent[cb];
    const V* sh = shift + (size_t)octant[cb] * Kp;
    const V* src = Psrc + ((size_t)(P * nrhs + r) * 2 + pol) * Kp;
    for (int m = threadIdx.x; m < Kp; m += blockDim.x) {
        const V z = sh[m], v = src[m];
        D[m] = CTraits<V>::make(v.x * z.x + v.y * z.y, v.y * z.x - v.x * z.y);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < Lp * Lc2; e += blockDim.x) {
        const int jp = e / Lp, it = e - jp * Lp;
        R ax = 0, ay = 0;
        for (int q = phT_ptr[jp]; q < phT_ptr[jp + 1]; ++q) {
            const R w = phT_w[q];
            const V d = D[phT_row[q] * Lp + it];
            ax = fma(w, d.x, ax);
            ay = fma(w, d.y, ay);
        }
        E[e] = CTraits<V>::make(ax, ay);
    }
    __syncthreads();
    const size_t off = ((size_t)cr * 2 + pol) * Kc;
    for (int e = threadIdx.x; e < Kc; e += blockDim.x) {
        const int jp = e / Lc, jt = e - jp * Lc;
        R ax = 0, ay = 0;
        for (int q = thT_ptr[jt]; q < thT_ptr[jt + 1]; ++q) {
            const R w = thT_w[q];
            const V v = E[jp * Lp + thT_row[q]];
            ax = fma(w, v.x, ax);
            ay = fma(w, v.y, ay);
        }
        const V bv = Bc[off + e];
        Ac[off + e] = CTraits<V>::make(bv.x + ax, bv.y + ay);
    }
}

}  // namespace mlf
