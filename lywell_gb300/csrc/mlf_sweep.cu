// Monostatic RCS sweep (gen_rcs_monostatica, main.f90:967-1089).
//
// mode 0 — the reference's sweep: angles phi_a in order, incidence
//   d = (-cos phi, -sin phi, 0) at theta = 90 deg, polarisation VV (z) or
//   HH (d x z normalised, ajustar_polariz main.f90:828-849), CGS on the FP64
//   operator warm-started from the previous angle's currents times
//   exp(-j k (d_a - d_{a-1}) . r_edge) (main.f90:1017-1022), backscatter
//   sigma(pi/2, phi_a).  The first guess is zero with d_0 = (-1, 0, 0).
// Blocks hold `block` angles; block <= 0 lets the autotuner choose it
// (mlf_autotune_block) among 8..128.
// mode 1 — batched: blocks of `block` angles solved together as one
//   multi-right-hand-side CGS on the FP64 operator (zero guesses, columns
//   retire independently).
// mode 2 — batched mixed precision: blocks solved by mlf_solve mode 1
//   (FP64 refinement around GMRES on the FP32 operator).
// mode 3 — batched mixed precision with the reference's warm starts: the
//   angles are dealt to the block's columns in contiguous runs (column q
//   sweeps angles [q * nrun, (q + 1) * nrun), nrun = ceil(nang / block)),
//   block k solves the k-th angle of every run, and each column starts from
//   its previous angle's currents phase-shifted as in mode 0.  Runs end
//   together except the last ones, so a block's live columns are a prefix.
// mode 4 — mode 3 with each column's start extrapolated from its two previous
//   angles: the currents are a slowly varying amplitude times the incident
//   phase, so with both shifted to the new direction, x0 = 2 x_{k-1} - x_{k-2}.
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

// x_i *= exp(-j kappa dR . e_centro_i)
__global__ void k_phase_shift(int N, const double* __restrict__ e_centro, double dx, double dy, double dz, double kappa,
                              double2* __restrict__ x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const double* e = e_centro + 3 * i;
    const double a = kappa * (dx * e[0] + dy * e[1] + dz * e[2]);
    double s, co;
    sincos(a, &s, &co);
    const double2 v = x[i];
    x[i] = make_double2(v.x * co + v.y * s, v.y * co - v.x * s);
}

// b = 2 a - b
__global__ void k_extrapolate(size_t n, const double2* __restrict__ a, double2* __restrict__ b) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        b[i] = make_double2(2. * a[i].x - b[i].x, 2. * a[i].y - b[i].y);
}

static void mono_dir(double phi, double* d) {
    d[0] = -std::cos(phi);
    d[1] = -std::sin(phi);
    d[2] = 0.;
}

static void mono_pol(const double* d, int hh, double2* p) {
    if (!hh) {
        p[0] = make_double2(0, 0); p[1] = make_double2(0, 0); p[2] = make_double2(1, 0);
        return;
    }
    // cross_productR(d, z) = (d2, -d1, 0), normalised
    const double v0 = d[1] * 1.0 - d[2] * 0.0, v1 = d[2] * 0.0 - d[0] * 1.0, v2 = d[0] * 0.0 - d[1] * 0.0;
    const double n = std::sqrt(v0 * v0 + v1 * v1 + v2 * v2);
    p[0] = make_double2(v0 / n, 0); p[1] = make_double2(v1 / n, 0); p[2] = make_double2(v2 / n, 0);
}

}  // namespace mlf

using namespace mlf;

extern "C" int mlf_monostatic(mlf_ctx* h, int nang, const double* phis, int hh, double ctte_re, double ctte_im,
                              double tol, int maxit, int precond_kind, int mode, int block, double* sigma, int* iters,
                              int* status_out) {
    DevScope ds;
    if (!h || nang <= 0 || !sigma || !iters || !status_out || maxit <= 0 || !(tol > 0) || mode < 0 || mode > 4)
        return MLF_E_ARG;
    Ctx* c = &h->c;
    if (!cuda_ok(c, cudaSetDevice(c->dev), "cudaSetDevice")) return MLF_E_CUDA;
    if ((precond_kind == 1 && !c->ilu_ok) || (precond_kind == 2 && !c->nearinv_ok) || precond_kind < 0 ||
        precond_kind > 2) {
        c->err = "requested preconditioner not built";
        return MLF_E_STATE;
    }
    const int N = c->N;
    const double2 ctte = make_double2(ctte_re, ctte_im);
    std::vector<double> ph(nang);
    const double dephi = 1. * PI / nang;
    for (int a = 0; a < nang; ++a) ph[a] = phis ? phis[a] : (a)*dephi;   // angphi = (ang-1)*dephi
    int st = MLF_OK;
    if (mode == 0) {
        double2 *b = nullptr, *x = nullptr, *g = nullptr;
        CK(ds.alloc(&b, N * sizeof(double2)));
        CK(ds.alloc(&x, N * sizeof(double2)));
        CK(ds.alloc(&g, N * sizeof(double2)));
        CK(cudaMemsetAsync(g, 0, N * sizeof(double2), c->stream));
        double prev[3] = {-1., 0., 0.};
        for (int a = 0; a < nang && !st; ++a) {
            double d[3];
            double2 pol[3];
            mono_dir(ph[a], d);
            k_phase_shift<<<(N + 255) / 256, 256, 0, c->stream>>>(N, c->de_centro, d[0] - prev[0], d[1] - prev[1],
                                                                  d[2] - prev[2], c->ph.kappa, g);
            mono_pol(d, hh, pol);
            if ((st = device_excitation(c, d, pol, ctte, 1, b))) break;
            double rr;
            if ((st = device_cgs(c, b, g, tol, maxit, 1, x, &iters[a], &rr, precond_kind, &status_out[a]))) break;
            const double th = PI / 2.;
            if ((st = device_rcs(c, x, pol, ctte, &th, &ph[a], 1, &sigma[a]))) break;
            CK(cudaMemcpyAsync(g, x, N * sizeof(double2), cudaMemcpyDeviceToDevice, c->stream));
            prev[0] = d[0]; prev[1] = d[1]; prev[2] = d[2];
        }
        return st;
    }
    int bsel = block;
    if (bsel <= 0) {
        // autotuned block: candidates up to the sweep length
        // modes 3 and 4: blocks small enough that every column sweeps a run of
        // at least four angles, so that most blocks start from extrapolated
        // warm starts
        std::vector<int> cand;
        const int bcap = mode >= 3 ? std::max(8, nang / 4) : nang;
        for (int b : {8, 16, 32, 64, 128})
            if (b <= bcap) cand.push_back(b);
        if (cand.empty()) cand.push_back(nang);
        int cols = 0;
        if ((st = autotune_block(c, cand.data(), (int)cand.size(), &bsel, &cols, nullptr, nullptr))) return st;
    }
    const int bs = std::max(1, std::min(bsel, nang));
    if (mode >= 3) {
        const int nrun = (nang + bs - 1) / bs;
        double2 *b = nullptr, *x = nullptr, *g = nullptr, *g2 = nullptr;
        CK(ds.alloc(&b, (size_t)N * bs * sizeof(double2)));
        CK(ds.alloc(&x, (size_t)N * bs * sizeof(double2)));
        CK(ds.alloc(&g, (size_t)N * bs * sizeof(double2)));    // previous angle's currents
        if (mode == 4) CK(ds.alloc(&g2, (size_t)N * bs * sizeof(double2)));   // the one before
        const size_t nbytes_col = (size_t)N * sizeof(double2);
        std::vector<double> dirs(3 * (size_t)bs), prev(3 * (size_t)bs), rr(bs);
        std::vector<double2> pols(3 * (size_t)bs);
        std::vector<int> it(bs), stc(bs);
        for (int k = 0; k < nrun && !st; ++k) {
            int nb = 0;
            while (nb < bs && nb * nrun + k < nang) ++nb;   // live columns: a prefix
            for (int q = 0; q < nb; ++q) {
                mono_dir(ph[q * nrun + k], &dirs[3 * q]);
                mono_pol(&dirs[3 * q], hh, &pols[3 * q]);
                if (k > 0)
                    k_phase_shift<<<(N + 255) / 256, 256, 0, c->stream>>>(
                        N, c->de_centro, dirs[3 * q] - prev[3 * q], dirs[3 * q + 1] - prev[3 * q + 1],
                        dirs[3 * q + 2] - prev[3 * q + 2], c->ph.kappa, g + (size_t)q * N);
                if (k > 1 && g2)
                    k_phase_shift<<<(N + 255) / 256, 256, 0, c->stream>>>(
                        N, c->de_centro, dirs[3 * q] - prev[3 * q], dirs[3 * q + 1] - prev[3 * q + 1],
                        dirs[3 * q + 2] - prev[3 * q + 2], c->ph.kappa, g2 + (size_t)q * N);
            }
            // mode 4: the two previous angles' currents, both phase-shifted to this
            // angle, extrapolated linearly (x0 = 2 x_{k-1} - x_{k-2}, into g2)
            const double2* x0 = k > 0 ? g : nullptr;
            if (k > 1 && g2) {
                k_extrapolate<<<4096, 256, 0, c->stream>>>((size_t)N * nb, g, g2);
                x0 = g2;
            }
            if ((st = device_excitation(c, dirs.data(), pols.data(), ctte, nb, b))) break;
            int outer = 0;
            if ((st = device_solve_mixed(c, b, x0, tol, maxit, nb, x, it.data(), rr.data(), precond_kind,
                                         stc.data(), 0.9 * tol, &outer)))
                break;
            // the block's backscatter in one launch (a CTA per column)
            std::vector<double> thq(nb, PI / 2.), phq(nb), sq(nb);
            for (int q = 0; q < nb; ++q) {
                const int a = q * nrun + k;
                iters[a] = it[q];
                status_out[a] = stc[q];
                phq[q] = ph[a];
            }
            if ((st = device_rcs_cols(c, x, (size_t)N, nb, pols.data(), ctte, thq.data(), phq.data(), sq.data())))
                break;
            for (int q = 0; q < nb; ++q) sigma[q * nrun + k] = sq[q];
            if (g2 && k > 0) std::swap(g, g2);   // g2 <- x_{k-1} in this angle's frame
            CK(cudaMemcpyAsync(g, x, nbytes_col * nb, cudaMemcpyDeviceToDevice, c->stream));
            std::copy(dirs.begin(), dirs.begin() + 3 * nb, prev.begin());
        }
        return st;
    }
    double2 *b = nullptr, *x = nullptr;
    CK(ds.alloc(&b, (size_t)N * bs * sizeof(double2)));
    CK(ds.alloc(&x, (size_t)N * bs * sizeof(double2)));
    std::vector<double> dirs(3 * (size_t)bs), rr(bs);
    std::vector<double2> pols(3 * (size_t)bs);
    for (int a0 = 0; a0 < nang && !st; a0 += bs) {
        const int nb = std::min(bs, nang - a0);
        for (int q = 0; q < nb; ++q) {
            mono_dir(ph[a0 + q], &dirs[3 * q]);
            mono_pol(&dirs[3 * q], hh, &pols[3 * q]);
        }
        if ((st = device_excitation(c, dirs.data(), pols.data(), ctte, nb, b))) break;
        if (mode == 1) {
            st = device_cgs(c, b, nullptr, tol, maxit, nb, x, &iters[a0], rr.data(), precond_kind, &status_out[a0]);
        } else {
            int outer = 0;
            st = device_solve_mixed(c, b, nullptr, tol, maxit, nb, x, &iters[a0], rr.data(), precond_kind,
                                    &status_out[a0], 0.9 * tol, &outer);
        }
        if (st) break;
        std::vector<double> thq(nb, PI / 2.);
        st = device_rcs_cols(c, x, (size_t)N, nb, pols.data(), ctte, thq.data(), &ph[a0], &sigma[a0]);
    }
    return st;
}
