// Z_mn of the RWG method of moments (Zmn_MoM, modMoM.f90:219-265; green,
// modGlobalMetod.f90:472-487): test point = centroid of each triangle of m,
// source = the 9 sub-centroids of each triangle of n, no singularity
// extraction; computed in FP64.  Shared by the near-field fill and the dense
// MoM operator.
#pragma once
#include <cuda_runtime.h>

#include "mlf_internal.h"

namespace mlf {

__device__ __forceinline__ double2 green(double w_smue, const double* a, const double* b) {
    const double d0 = a[0] - b[0], d1 = a[1] - b[1], d2 = a[2] - b[2];
    const double r = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
    double s, co;
    sincos(w_smue * r, &s, &co);
    const double ir = 1.0 / r;
    return make_double2(co * ir, -s * ir);
}

__device__ __forceinline__ double2 zmn_mom(int m, int n, const double* __restrict__ t_baric,
                                           const double* __restrict__ t_baric_sub,
                                           const double* __restrict__ p_coord, const int* __restrict__ e_t,
                                           const int* __restrict__ e_po, const double* __restrict__ e_long, double w,
                                           double w_smue, double c72) {
    const double* cpm = t_baric + 3 * e_t[2 * m];
    const double* cmm = t_baric + 3 * e_t[2 * m + 1];
    const double* vpm = p_coord + 3 * e_po[2 * m];
    const double* vmm = p_coord + 3 * e_po[2 * m + 1];
    const double lm = e_long[m];
    const int tpn = e_t[2 * n], tmn = e_t[2 * n + 1];
    const double* vpn = p_coord + 3 * e_po[2 * n];
    const double* vmn = p_coord + 3 * e_po[2 * n + 1];
    double2 AP[3] = {{0, 0}, {0, 0}, {0, 0}}, AM[3] = {{0, 0}, {0, 0}, {0, 0}};
    double2 PhiP = {0, 0}, PhiM = {0, 0};
    for (int i = 0; i < 9; ++i) {
        const double* sp = t_baric_sub + 27 * (size_t)tpn + 3 * i;
        const double* sm = t_baric_sub + 27 * (size_t)tmn + 3 * i;
        const double2 g11 = green(w_smue, cpm, sp), g12 = green(w_smue, cpm, sm);
        const double2 g21 = green(w_smue, cmm, sp), g22 = green(w_smue, cmm, sm);
        for (int d = 0; d < 3; ++d) {
            const double r1 = sp[d] - vpn[d], r2 = vmn[d] - sm[d];
            AP[d].x += g11.x * r1 + g12.x * r2; AP[d].y += g11.y * r1 + g12.y * r2;
            AM[d].x += g21.x * r1 + g22.x * r2; AM[d].y += g21.y * r1 + g22.y * r2;
        }
        PhiP.x += g11.x - g12.x; PhiP.y += g11.y - g12.y;
        PhiM.x += g21.x - g22.x; PhiM.y += g21.y - g22.y;
    }
    const double ln = e_long[n];
    const double fa = ((MU / PI) * c72) * ln;
    const double den = ((36 * PI) * w) * EPSI;
    // Phi = -Phi*l_n / (j den) = (-Im*l_n/den... ) written out
    const double tPx = -PhiP.x * ln, tPy = -PhiP.y * ln, tMx = -PhiM.x * ln, tMy = -PhiM.y * ln;
    const double2 P2 = make_double2(tPy / den, -tPx / den), M2 = make_double2(tMy / den, -tMx / den);
    double2 s = {0, 0};
    for (int d = 0; d < 3; ++d) {
        const double a1 = cpm[d] - vpm[d], a2 = -cmm[d] + vmm[d];
        s.x += AP[d].x * fa * a1 + AM[d].x * fa * a2;
        s.y += AP[d].y * fa * a1 + AM[d].y * fa * a2;
    }
    const double fz = (0.5 * w) * lm;
    const double2 PintA = make_double2(-fz * s.y, fz * s.x);
    const double2 PintPhi = make_double2(lm * (M2.x - P2.x), lm * (M2.y - P2.y));
    return make_double2(PintPhi.x + PintA.x, PintPhi.y + PintA.y);
}

}  // namespace mlf
