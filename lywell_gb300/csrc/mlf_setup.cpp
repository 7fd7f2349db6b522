// Host-side set-up of the MLFMA solve: RWG basis, octree, sampling grids,
// far/near interaction lists, interpolation tables, ILU(0) factorisation and
// the level schedule of its triangular sweeps.
//
// Everything here is combinatorial or O(N log N); the O(N^2) searches of the
// reference (node dedup, shared-edge search, box-pair scans) are replaced by
// hashing with identical outcomes.  Floating-point steps that decide box
// membership or table values keep the reference's operation order, including
// its single-precision literals.  Compiled with -ffp-contract=off.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <unordered_map>

#include "mlf_internal.h"

namespace mlf {

Phys phys_from_lambda(double lambda) {
    // setlambda, modGlobalParam.f90:52-61
    Phys p;
    p.vp = 1.0 / std::sqrt(MU * EPSI);
    p.lambda = lambda;
    p.w = 2. * PI * p.vp / lambda;
    p.kappa = 2. * PI / lambda;
    p.smue = std::sqrt(MU * EPSI);
    return p;
}

// ---------------------------------------------------------------------------
// special functions
// ---------------------------------------------------------------------------

// Spherical Bessel j_n and y_n, n = 0..nmax, x > 0.  y_n by upward recurrence.
// j_n by upward recurrence when nmax <= x, else by Miller's backward
// recurrence started above max(nmax, x) and scaled to j_0 (or j_1 when j_0 is
// the smaller of the two, i.e. near a zero of sin x).
void sph_bessel(int nmax, double x, double* j, double* y) {
    const double sx = std::sin(x), cx = std::cos(x);
    const double j0 = sx / x, j1 = sx / (x * x) - cx / x;
    y[0] = -cx / x;
    if (nmax >= 1) y[1] = -cx / (x * x) - sx / x;
    for (int n = 1; n < nmax; ++n) y[n + 1] = (2.0 * n + 1.0) / x * y[n] - y[n - 1];
    if ((double)nmax <= x) {
        j[0] = j0;
        if (nmax >= 1) j[1] = j1;
        for (int n = 1; n < nmax; ++n) j[n + 1] = (2.0 * n + 1.0) / x * j[n] - j[n - 1];
        return;
    }
    const int start = std::max(nmax, (int)x) + 30 + (int)(10.0 * std::cbrt(x + 1.0));
    double hi = 0.0, cur = 1e-280;
    for (int n = start; n >= 1; --n) {
        const double lo = (2.0 * n + 1.0) / x * cur - hi;
        hi = cur;
        cur = lo;
        if (n - 1 <= nmax) j[n - 1] = cur;
        if (std::fabs(cur) > 1e250) {
            cur *= 1e-250;
            hi *= 1e-250;
            for (int q = std::max(n - 1, 0); q <= nmax; ++q) j[q] *= 1e-250;
        }
    }
    const double s = std::fabs(j0) > std::fabs(j1) ? j0 / j[0] : j1 / j[1];
    for (int n = 0; n <= nmax; ++n) j[n] *= s;
}

// (n! / (i! (n-i)!))^2 with the factorials formed as sequential double
// products, the way legendre/factorial do it (modGlobalMetod.f90:988-1015).
void binomial_squares(int nmax, std::vector<double>& out) {
    std::vector<double> fact(nmax + 1);
    for (int x = 0; x <= nmax; ++x) {
        double r = 1.;
        for (int i = 1; i <= x; ++i) r = r * i;
        fact[x] = r;
    }
    out.assign((size_t)(nmax + 1) * (nmax + 1), 0.0);
    for (int n = 0; n <= nmax; ++n)
        for (int i = 0; i <= n; ++i) {
            const double c = fact[n] / (fact[i] * fact[n - i]);
            out[(size_t)n * (nmax + 1) + i] = c * c;
        }
}

// ---------------------------------------------------------------------------
// RWG basis
// ---------------------------------------------------------------------------

namespace {

struct Vec3Hash {
    size_t operator()(const std::array<uint64_t, 3>& k) const {
        uint64_t h = k[0] * 0x9E3779B97F4A7C15ull;
        h ^= k[1] + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
        h ^= k[2] + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
        return (size_t)h;
    }
};

uint64_t dbits(double v) {
    v = v + 0.0;  // -0.0 -> +0.0: exact equality as in the reference's comparisons
    uint64_t u;
    std::memcpy(&u, &v, 8);
    return u;
}

}  // namespace

}  // namespace mlf

using namespace mlf;

extern "C" int mlf_rwg_build(const double* tris, int T, int* N_out, int* P_out, double* p_coord,
                             int* t_p, int* e_p, int* e_t, int* e_po, double* e_long,
                             double* e_centro, double* t_area, double* t_baric,
                             double* t_baric_sub) {
    if (!tris || T <= 0 || !N_out || !P_out) return MLF_E_ARG;
    // node deduplication by exact coordinates (limpiarnodos,
    // modReadStl.f90:1444-1533); ids in first-occurrence order
    std::unordered_map<std::array<uint64_t, 3>, int, Vec3Hash> nodes;
    nodes.reserve((size_t)T * 2);
    std::vector<int> tp((size_t)3 * T);
    std::vector<double> pc;
    for (int t = 0; t < T; ++t)
        for (int k = 0; k < 3; ++k) {
            const double* v = tris + 9 * (size_t)t + 3 * k;
            std::array<uint64_t, 3> key{dbits(v[0]), dbits(v[1]), dbits(v[2])};
            auto it = nodes.find(key);
            int id;
            if (it == nodes.end()) {
                id = (int)(pc.size() / 3);
                nodes.emplace(key, id);
                pc.insert(pc.end(), {v[0], v[1], v[2]});
            } else {
                id = it->second;
            }
            tp[3 * (size_t)t + k] = id;
        }
    const int P = (int)(pc.size() / 3);
    // edge list (llenar_lados, modRWG.f90:8-29): per triangle (1,2),(1,3),(2,3);
    // an edge is made at the first occurrence of a pair that occurs again
    // (Buscar_L_Comun / llenar_todo, modRWG.f90:32-131)
    const int M = 3 * T;
    std::vector<int> la(M), lb(M);
    for (int t = 0; t < T; ++t) {
        la[3 * t] = tp[3 * t]; lb[3 * t] = tp[3 * t + 1];
        la[3 * t + 1] = tp[3 * t]; lb[3 * t + 1] = tp[3 * t + 2];
        la[3 * t + 2] = tp[3 * t + 1]; lb[3 * t + 2] = tp[3 * t + 2];
    }
    // sides sorted by (node pair, side index): equal pairs are adjacent, in side order
    std::vector<std::pair<uint64_t, int>> ks(M);
    for (int i = 0; i < M; ++i) {
        const uint64_t a = (uint64_t)std::min(la[i], lb[i]), b = (uint64_t)std::max(la[i], lb[i]);
        ks[i] = {(a << 32) | b, i};
    }
    std::sort(ks.begin(), ks.end());
    std::vector<std::pair<int, int>> pairs;
    pairs.reserve(M / 2);
    for (int s = 0; s < M;) {
        int e = s;
        while (e + 1 < M && ks[e + 1].first == ks[s].first) ++e;
        for (int q = s; q + 1 <= e; q += 2) pairs.emplace_back(ks[q].second, ks[q + 1].second);
        s = e + 1;
    }
    std::sort(pairs.begin(), pairs.end());
    const int N = (int)pairs.size();
    *N_out = N;
    *P_out = P;
    if (!p_coord) return MLF_OK;
    std::memcpy(p_coord, pc.data(), sizeof(double) * pc.size());
    for (int i = 0; i < 3 * T; ++i) t_p[i] = tp[i] + 1;
    for (int e = 0; e < N; ++e) {
        const int i = pairs[e].first, j = pairs[e].second;
        const int x = i / 3, y = j / 3;
        const int p1 = la[i], p2 = lb[i];
        e_p[2 * e] = p1 + 1;
        e_p[2 * e + 1] = p2 + 1;
        e_t[2 * e] = x + 1;
        e_t[2 * e + 1] = y + 1;
        for (int s = 0; s < 2; ++s) {
            const int tri = s == 0 ? x : y;
            const int* t3 = &tp[3 * (size_t)tri];
            int o;
            if (t3[0] != p1 && t3[0] != p2) o = t3[0];
            else if (t3[1] != p1 && t3[1] != p2) o = t3[1];
            else o = t3[2];
            e_po[2 * e + s] = o + 1;
        }
        // parametros_rwg, modRWG.f90:161-164
        const double* a = &pc[3 * (size_t)p1];
        const double* b = &pc[3 * (size_t)p2];
        const double d0 = a[0] - b[0], d1 = a[1] - b[1], d2 = a[2] - b[2];
        e_long[e] = std::sqrt((d0 * d0 + d1 * d1) + d2 * d2);
        for (int k = 0; k < 3; ++k) e_centro[3 * e + k] = 0.5 * (a[k] + b[k]);
    }
    // hallar_geometria_rwg, modRWG.f90:270-328 (single-precision 1/3, 2/3)
    const double f13 = (double)(1.0f / 3.0f), f23 = (double)(2.0f / 3.0f);
    static const int trip[9][3] = {{1, 4, 9}, {4, 5, 10}, {5, 2, 6}, {6, 10, 7}, {7, 8, 3},
                                   {7, 8, 10}, {8, 9, 10}, {9, 4, 10}, {5, 6, 10}};
    for (int t = 0; t < T; ++t) {
        const double* p1 = &pc[3 * (size_t)tp[3 * t]];
        const double* p2 = &pc[3 * (size_t)tp[3 * t + 1]];
        const double* p3 = &pc[3 * (size_t)tp[3 * t + 2]];
        double v[11][3];
        for (int k = 0; k < 3; ++k) {
            const double bc = f13 * ((p1[k] + p2[k]) + p3[k]);
            t_baric[3 * t + k] = bc;
            v[1][k] = p1[k]; v[2][k] = p2[k]; v[3][k] = p3[k];
            v[4][k] = p1[k] + f13 * (p2[k] - p1[k]);
            v[5][k] = p1[k] + f23 * (p2[k] - p1[k]);
            v[6][k] = p2[k] + f13 * (p3[k] - p2[k]);
            v[7][k] = p2[k] + f23 * (p3[k] - p2[k]);
            v[8][k] = p3[k] + f13 * (p1[k] - p3[k]);
            v[9][k] = p3[k] + f23 * (p1[k] - p3[k]);
            v[10][k] = bc;
        }
        for (int s = 0; s < 9; ++s)
            for (int k = 0; k < 3; ++k)
                t_baric_sub[27 * (size_t)t + 3 * s + k] =
                    f13 * ((v[trip[s][0]][k] + v[trip[s][1]][k]) + v[trip[s][2]][k]);
        double ba[3], ca[3];
        for (int k = 0; k < 3; ++k) { ba[k] = p1[k] - p2[k]; ca[k] = p1[k] - p3[k]; }
        const double c0 = ba[1] * ca[2] - ba[2] * ca[1];
        const double c1 = ba[2] * ca[0] - ba[0] * ca[2];
        const double c2 = ba[0] * ca[1] - ba[1] * ca[0];
        t_area[t] = 0.5 * std::sqrt((c0 * c0 + c1 * c1) + c2 * c2);
    }
    return MLF_OK;
}

namespace mlf {

// ---------------------------------------------------------------------------
// octree
// ---------------------------------------------------------------------------

namespace {

// llenar_kappas, modMLFMA.f90:453-495: midpoint theta (L) x phi (2L), theta
// fastest; weight (cos((k-1)dth) - cos(k dth)) dphi.
void sampling(Level& L) {
    const int K = L.K;
    L.kap.resize(3 * (size_t)K); L.ath.resize(3 * (size_t)K); L.aph.resize(3 * (size_t)K);
    L.ang.resize(2 * (size_t)K); L.wq.resize(K);
    const double dphi = 2. * PI / L.nph, dth = PI / L.nth;
    int q = 0;
    for (int j = 1; j <= L.nph; ++j) {
        const double phi = (dphi / 2.) * ((2 * j) - 1);
        const double sp = std::sin(phi), cp = std::cos(phi);
        for (int k = 1; k <= L.nth; ++k, ++q) {
            const double th = (dth / 2.) * ((2 * k) - 1);
            const double st = std::sin(th), ct = std::cos(th);
            L.kap[3 * q] = st * cp; L.kap[3 * q + 1] = st * sp; L.kap[3 * q + 2] = ct;
            L.ath[3 * q] = ct * cp; L.ath[3 * q + 1] = ct * sp; L.ath[3 * q + 2] = -st;
            L.aph[3 * q] = -sp; L.aph[3 * q + 1] = cp; L.aph[3 * q + 2] = 0.;
            L.ang[2 * q] = th; L.ang[2 * q + 1] = phi;
            L.wq[q] = (std::cos((k - 1) * dth) - std::cos(k * dth)) * dphi;
        }
    }
}

// Nearest sample index (1-based) on an increasing midpoint grid by the
// reference's bisection, then its two neighbours with wrap-around at both
// ends (hallarKcercanos, modMLFMA.f90:1096-1315).
void nearest3(const double* grid, int stride, int n, double x, long out[3]) {
    auto g = [&](long i) { return grid[(size_t)(i - 1) * stride]; };
    long lo = 1, hi = n, mid;
    for (;;) {
        mid = (lo + hi) / 2;
        const double v = g(mid);
        if (mid == lo || mid == hi) {
            mid = std::fabs(x - g(lo)) < std::fabs(x - g(hi)) ? lo : hi;
            break;
        }
        if (v == x) break;
        if (v > x) hi = mid;
        else if (v < x) lo = mid;
    }
    long below, above;
    if (mid == 1) { below = n; above = 2; }
    else if (mid == n) { below = n - 1; above = 1; }
    else { below = mid - 1; above = mid + 1; }
    out[0] = mid; out[1] = below; out[2] = above;
}

// 3-point Lagrange weights (Wlagrange3, modMLFMA.f90:1318-1341)
void lagrange3(double x, const double m[3], double W[3]) {
    for (int i = 0; i < 3; ++i) {
        double w = 1.;
        for (int j = 0; j < 3; ++j)
            if (j != i) w = w * ((x - m[j]) / (m[i] - m[j]));
        W[i] = w;
    }
}

// llenarMinterp, modMLFMA.f90:998-1092: 9 taps per coarse sample, weight
// Wtheta(m2) * Wphi(m1) on child sample (phi_m1, theta_m2).
void interp_table(const Level& Lc /*coarse*/, const Level& Lf /*fine*/, std::vector<double>& iw,
                  std::vector<int>& iidx) {
    iw.resize(9 * (size_t)Lc.K);
    iidx.resize(9 * (size_t)Lc.K);
    const int nth = Lf.nth;
    for (int i = 0; i < Lc.K; ++i) {
        const double xt = Lc.ang[2 * i], xp = Lc.ang[2 * i + 1];
        long ph[3], th[3];
        nearest3(&Lf.ang[1], 2 * nth, Lf.nph, xp, ph);   // phi of sample (p-1)*nth+1
        nearest3(&Lf.ang[0], 2, nth, xt, th);            // theta of sample t
        const double mt[3] = {Lf.ang[2 * (th[0] - 1)], Lf.ang[2 * (th[1] - 1)], Lf.ang[2 * (th[2] - 1)]};
        const double mp[3] = {Lf.ang[2 * ((ph[0] - 1) * nth) + 1], Lf.ang[2 * ((ph[1] - 1) * nth) + 1],
                              Lf.ang[2 * ((ph[2] - 1) * nth) + 1]};
        double Wt[3], Wp[3];
        lagrange3(xt, mt, Wt);
        lagrange3(xp, mp, Wp);
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                iw[9 * (size_t)i + 3 * a + b] = Wt[b] * Wp[a];
                iidx[9 * (size_t)i + 3 * a + b] = (int)(nth * (ph[a] - 1) + th[b]) - 1;
            }
    }
}

// Separable form of the same stencil: for each coarse theta row the three
// fine theta rows (posT, posTmen, posTmay) and their Lagrange weights, for
// each coarse phi column the three fine phi columns and weights; the 9-tap
// weight of interp_table is exactly wth[a] * wph[b].
void separable_tables(const Level& Lc, const Level& Lf, Level& out) {
    const int Lt = Lc.nth, Lp2 = Lc.nph, nth = Lf.nth;
    out.sth.assign(3 * Lt, 0); out.wth.assign(3 * Lt, 0);
    out.sph.assign(3 * Lp2, 0); out.wph.assign(3 * Lp2, 0);
    for (int it = 0; it < Lt; ++it) {
        const double xt = Lc.ang[2 * it];           // theta of coarse sample it (phi column 0)
        long th[3];
        nearest3(&Lf.ang[0], 2, nth, xt, th);
        const double mt[3] = {Lf.ang[2 * (th[0] - 1)], Lf.ang[2 * (th[1] - 1)], Lf.ang[2 * (th[2] - 1)]};
        double Wt[3];
        lagrange3(xt, mt, Wt);
        for (int a = 0; a < 3; ++a) { out.sth[3 * it + a] = (int)th[a] - 1; out.wth[3 * it + a] = Wt[a]; }
    }
    for (int ip = 0; ip < Lp2; ++ip) {
        const double xp = Lc.ang[2 * ((size_t)ip * Lt) + 1];
        long ph[3];
        nearest3(&Lf.ang[1], 2 * nth, Lf.nph, xp, ph);
        const double mp[3] = {Lf.ang[2 * ((ph[0] - 1) * nth) + 1], Lf.ang[2 * ((ph[1] - 1) * nth) + 1],
                              Lf.ang[2 * ((ph[2] - 1) * nth) + 1]};
        double Wp[3];
        lagrange3(xp, mp, Wp);
        for (int b = 0; b < 3; ++b) { out.sph[3 * ip + b] = (int)ph[b] - 1; out.wph[3 * ip + b] = Wp[b]; }
    }
    auto transpose = [](const std::vector<int>& idx, const std::vector<double>& w, int ncoarse, int nfine,
                        std::vector<int>& ptr, std::vector<int>& row, std::vector<double>& ww) {
        ptr.assign(nfine + 1, 0);
        for (int e = 0; e < 3 * ncoarse; ++e) ptr[idx[e] + 1]++;
        for (int q = 0; q < nfine; ++q) ptr[q + 1] += ptr[q];
        row.assign(3 * ncoarse, 0);
        ww.assign(3 * ncoarse, 0);
        std::vector<int> fill(ptr.begin(), ptr.end() - 1);
        for (int e = 0; e < 3 * ncoarse; ++e) {
            row[fill[idx[e]]] = e / 3;
            ww[fill[idx[e]]] = w[e];
            fill[idx[e]]++;
        }
    };
    transpose(out.sth, out.wth, Lt, Lf.nth, out.thT_ptr, out.thT_row, out.thT_w);
    transpose(out.sph, out.wph, Lp2, Lf.nph, out.phT_ptr, out.phT_row, out.phT_w);
}

struct Builder {
    Ctx* c;
    std::vector<int> leaf_bases, leaf_ptr;
    std::vector<int> work;

    // geomMLFMA / dividir_en_8_hijos / buscarFuncBases (modMLFMA.f90:497-833):
    // a basis goes to the first child, in the fixed child order, whose closed
    // box holds its edge centre; empty children are not stored.
    void split(const double centre[3], double side, std::vector<int>& bases, int level) {
        if (level == c->nlev) return;
        static const int sx[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
        static const int sy[8] = {-1, 1, -1, 1, -1, 1, -1, 1};
        static const int sz[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
        const double half = side / 2., quarter = side / 4.;
        Level& ch = c->lv[level + 1];
        double cc[8][3], lo[8][3], hi[8][3];
        for (int i = 0; i < 8; ++i) {
            cc[i][0] = sx[i] < 0 ? centre[0] - quarter : centre[0] + quarter;
            cc[i][1] = sy[i] < 0 ? centre[1] - quarter : centre[1] + quarter;
            cc[i][2] = sz[i] < 0 ? centre[2] - quarter : centre[2] + quarter;
            const double q = half / 2.;
            for (int d = 0; d < 3; ++d) { hi[i][d] = cc[i][d] + q; lo[i][d] = cc[i][d] - q; }
        }
        // one pass: each basis to the first child (in the fixed order) whose
        // closed box holds it -- what filtering child by child gives -- in
        // the order of `bases`
        std::array<std::vector<int>, 8> kids;
        for (int b : bases) {
            const double* e = &c->e_centro[3 * (size_t)b];
            for (int i = 0; i < 8; ++i) {
                if (e[0] <= hi[i][0] && e[0] >= lo[i][0] && e[1] <= hi[i][1] && e[1] >= lo[i][1] &&
                    e[2] <= hi[i][2] && e[2] >= lo[i][2]) {
                    kids[i].push_back(b);
                    break;
                }
            }
        }
        for (int i = 0; i < 8; ++i) {
            std::vector<int>& found = kids[i];
            if (found.empty()) continue;
            ch.centre.insert(ch.centre.end(), cc[i], cc[i] + 3);
            ch.parent.push_back(cur_parent[level]);
            ch.octant.push_back(i);
            ch.nb++;
            if (level + 1 == c->nlev) {
                leaf_bases.insert(leaf_bases.end(), found.begin(), found.end());
                leaf_ptr.push_back((int)leaf_bases.size());
            }
            const int saved = cur_parent[level + 1];
            cur_parent[level + 1] = ch.nb - 1;
            split(cc[i], half, found, level + 1);
            cur_parent[level + 1] = saved;
        }
    }
    int cur_parent[33]{};
};

// f(i) for i in [0, n) on up to 16 host threads in contiguous ranges; the
// calls must be independent
template <class F>
void parallel_for(int n, F f) {
    const int nt = (int)std::min<unsigned>(16, std::max(1u, std::thread::hardware_concurrency()));
    if (nt == 1 || n < 4096) {
        for (int i = 0; i < n; ++i) f(i);
        return;
    }
    // chunk t of nt covers [n t / nt, n (t + 1) / nt); chunks run on threads,
    // and any chunk whose thread could not be created (a process or container
    // thread limit: std::system_error) runs here, so no exception crosses the
    // C ABI and the result does not depend on how many threads started
    auto chunk = [&](int t) {
        const int i0 = (int)((long long)n * t / nt), i1 = (int)((long long)n * (t + 1) / nt);
        for (int i = i0; i < i1; ++i) f(i);
    };
    std::vector<std::thread> th;
    th.reserve(nt);
    int started = 0;
    for (; started < nt; ++started) {
        try {
            th.emplace_back(chunk, started);
        } catch (...) {
            break;
        }
    }
    for (int t = started; t < nt; ++t) chunk(t);
    for (auto& x : th) x.join();
}

inline long long cell_key(int a, int b, int cc) {
    return ((long long)(a + 1) << 42) | ((long long)(b + 1) << 21) | (long long)(cc + 1);
}

}  // namespace

int build_octree(Ctx* c) {
    const int N = c->N;
    const double lambda = c->ph.lambda;
    // root cube: bounding box of edge centres (limites_dispersor,
    // modGlobalMetod.f90:386-434) plus lambda/10000 (modMLFMA.f90:160-188)
    int lim[6] = {0, 0, 0, 0, 0, 0};
    const double* ec = c->e_centro.data();
    for (int i = 1; i < N; ++i) {
        const double* p = ec + 3 * i;
        if (p[0] > ec[3 * lim[0]]) lim[0] = i;
        if (p[0] < ec[3 * lim[1]]) lim[1] = i;
        if (p[1] > ec[3 * lim[2] + 1]) lim[2] = i;
        if (p[1] < ec[3 * lim[3] + 1]) lim[3] = i;
        if (p[2] > ec[3 * lim[4] + 2]) lim[4] = i;
        if (p[2] < ec[3 * lim[5] + 2]) lim[5] = i;
    }
    const double maxX = ec[3 * lim[0]], minX = ec[3 * lim[1]];
    const double maxY = ec[3 * lim[2] + 1], minY = ec[3 * lim[3] + 1];
    const double maxZ = ec[3 * lim[4] + 2], minZ = ec[3 * lim[5] + 2];
    const double dX = maxX - minX, dY = maxY - minY, dZ = maxZ - minZ;
    double side;
    if (dX >= dY && dX >= dZ) side = dX;
    else if (dY >= dX && dY >= dZ) side = dY;
    else side = dZ;
    side = side + lambda / 10000.;
    c->root_centre[0] = 0.5 * (maxX + minX);
    c->root_centre[1] = 0.5 * (maxY + minY);
    c->root_centre[2] = 0.5 * (maxZ + minZ);
    c->root_side = side;
    // nivel_max = ceiling(1 + log10(side/(ladomax*lambda))/log10(2.)), with
    // log10(2.) of a single-precision argument (modMLFMA.f90:189)
    const double log10_2f = (double)std::log10(2.0f);
    const int nl = (int)std::ceil(1. + (std::log10(side / (c->ladomax * lambda)) / log10_2f));
    c->nlev = nl;
    if (nl <= 3) {
        c->err = "body too small electrically for MLFMA (nivel_max <= 3)";
        return MLF_E_TOO_SMALL;
    }
    if (nl > 20) {
        c->err = "more than 20 octree levels";
        return MLF_E_ARG;
    }
    // per-level multipoles L = floor(kd + 6 (kd)^(1/3)), d = sqrt(3.) side with
    // sqrt(3.) and 1./3. in single precision (modMLFMA.f90:200-218)
    const double s3 = (double)std::sqrt(3.0f), third = (double)(1.0f / 3.0f);
    for (int i = 1; i <= nl; ++i) {
        Level& L = c->lv[i];
        L.side = side / std::ldexp(1.0, i - 1);
        const double kd = (2. * PI / lambda) * (s3 * L.side);
        L.L = (int)std::floor(kd + 6 * std::pow(kd, third));
        L.nth = L.L;
        L.nph = 2 * L.L;
        L.K = L.nth * L.nph;
        if (i >= 3) sampling(L);
    }
    // boxes
    Builder B;
    B.c = c;
    Level& root = c->lv[1];
    root.nb = 1;
    root.centre.assign(c->root_centre, c->root_centre + 3);
    root.parent.push_back(-1);
    root.octant.push_back(0);
    std::vector<int> all(N);
    for (int i = 0; i < N; ++i) all[i] = i;
    B.leaf_ptr.push_back(0);
    B.cur_parent[1] = 0;
    B.split(c->root_centre, side, all, 1);
    c->box_bases = std::move(B.leaf_bases);
    c->box_ptr = std::move(B.leaf_ptr);
    Level& leaf = c->lv[nl];
    c->box_of.assign(N, -1);
    for (int b = 0; b < leaf.nb; ++b)
        for (int t = c->box_ptr[b]; t < c->box_ptr[b + 1]; ++t) c->box_of[c->box_bases[t]] = b;
    for (int i = 1; i < nl; ++i) {
        Level& L = c->lv[i];
        const Level& Lc = c->lv[i + 1];
        L.child_ptr.assign(L.nb + 1, 0);
        for (int b = 0; b < Lc.nb; ++b) L.child_ptr[Lc.parent[b] + 1]++;
        for (int b = 0; b < L.nb; ++b) L.child_ptr[b + 1] += L.child_ptr[b];
    }
    // far / near lists (llenar_functransf, modMLFMA.f90:835-960).  Candidate
    // partners of box i are the children of the 27 neighbours of i's parent;
    // they are visited in ascending box index, as the reference's j loop, and
    // classified with its tests |dc_parent| < 2 s_p - tol, |dc| >= 2 s - tol.
    const double tol = lambda / 100.;
    const double ox = c->root_centre[0] - side / 2., oy = c->root_centre[1] - side / 2.,
                 oz = c->root_centre[2] - side / 2.;
    std::vector<std::vector<int>> cells(nl + 1);
    for (int n = 2; n <= nl; ++n) {
        Level& L = c->lv[n];
        cells[n].resize(3 * (size_t)L.nb);
        for (int b = 0; b < L.nb; ++b) {
            cells[n][3 * b] = (int)std::floor((L.centre[3 * b] - ox) / L.side);
            cells[n][3 * b + 1] = (int)std::floor((L.centre[3 * b + 1] - oy) / L.side);
            cells[n][3 * b + 2] = (int)std::floor((L.centre[3 * b + 2] - oz) / L.side);
        }
    }
    c->near_ptr.assign(1, 0);
    c->near_bases.clear();
    c->nbox_ptr.assign(1, 0);
    c->nbox_list.clear();
    for (int n = 3; n <= nl; ++n) {
        Level& L = c->lv[n];
        const Level& Lp = c->lv[n - 1];
        // parent cells: a dense grid (2^(n-2) per axis) while it has at most
        // 2^21 cells, else a hash map
        const long long G = 1LL << (n - 2);
        const bool dense = G * G * G <= (1LL << 21);
        std::vector<int> pgrid;
        std::unordered_map<long long, int> pcell;
        if (dense) {
            pgrid.assign((size_t)(G * G * G), -1);
            for (int b = 0; b < Lp.nb; ++b) {
                const int* q = &cells[n - 1][3 * b];
                if (q[0] >= 0 && q[0] < G && q[1] >= 0 && q[1] < G && q[2] >= 0 && q[2] < G)
                    pgrid[(size_t)((q[0] * G + q[1]) * G + q[2])] = b;
                else
                    pcell[cell_key(q[0], q[1], q[2])] = b;   // outside the grid: kept in the map
            }
        } else {
            pcell.reserve(2 * (size_t)Lp.nb);
            for (int b = 0; b < Lp.nb; ++b)
                pcell[cell_key(cells[n - 1][3 * b], cells[n - 1][3 * b + 1], cells[n - 1][3 * b + 2])] = b;
        }
        auto parent_at = [&](int x, int y, int z) -> int {
            if (dense && x >= 0 && x < G && y >= 0 && y < G && z >= 0 && z < G)
                return pgrid[(size_t)((x * G + y) * G + z)];
            if (pcell.empty()) return -1;
            auto it = pcell.find(cell_key(x, y, z));
            return it == pcell.end() ? -1 : it->second;
        };
        // translation index by cell offset (children of the parent's neighbours
        // lie within +-3 cells; numbered in order of first appearance)
        constexpr int OFF = 8, SPAN = 2 * OFF + 1;
        std::vector<int> tid_lut(SPAN * SPAN * SPAN, -1);
        std::unordered_map<long long, int> tid_of;   // offsets beyond the table (not expected)
        L.far_ptr.assign(1, 0);
        L.far_src.clear();
        L.far_tid.clear();
        L.rab.clear();
        std::vector<int> cand;
        for (int i = 0; i < L.nb; ++i) {
            const int ip = L.parent[i];
            cand.clear();
            const int* pc = &cells[n - 1][3 * ip];
            // children of distinct parents are disjoint contiguous ranges, so
            // ordering the ranges by their start orders the candidates
            int nrg = 0;
            std::array<int, 27> rg;
            for (int dx = -1; dx <= 1; ++dx)
                for (int dy = -1; dy <= 1; ++dy)
                    for (int dz = -1; dz <= 1; ++dz) {
                        const int pb = parent_at(pc[0] + dx, pc[1] + dy, pc[2] + dz);
                        if (pb >= 0 && Lp.child_ptr[pb + 1] > Lp.child_ptr[pb]) rg[nrg++] = pb;
                    }
            std::sort(rg.begin(), rg.begin() + nrg,
                      [&](int a, int b2) { return Lp.child_ptr[a] < Lp.child_ptr[b2]; });
            for (int q = 0; q < nrg; ++q)
                for (int j = Lp.child_ptr[rg[q]]; j < Lp.child_ptr[rg[q] + 1]; ++j) cand.push_back(j);
            for (int j : cand) {
                const int jp = L.parent[j];
                double rp[3], rh[3];
                for (int d = 0; d < 3; ++d) rp[d] = Lp.centre[3 * ip + d] - Lp.centre[3 * jp + d];
                const double np_ = std::sqrt(rp[0] * rp[0] + rp[1] * rp[1] + rp[2] * rp[2]);
                if (!(np_ < (2 * Lp.side - tol))) continue;
                for (int d = 0; d < 3; ++d) rh[d] = L.centre[3 * i + d] - L.centre[3 * j + d];
                const double nh = std::sqrt(rh[0] * rh[0] + rh[1] * rh[1] + rh[2] * rh[2]);
                if (nh >= (2 * L.side - tol)) {
                    const int ox_ = cells[n][3 * i] - cells[n][3 * j] + OFF,
                              oy_ = cells[n][3 * i + 1] - cells[n][3 * j + 1] + OFF,
                              oz_ = cells[n][3 * i + 2] - cells[n][3 * j + 2] + OFF;
                    const bool in_lut = ox_ >= 0 && ox_ < SPAN && oy_ >= 0 && oy_ < SPAN && oz_ >= 0 && oz_ < SPAN;
                    int* slot = in_lut ? &tid_lut[(ox_ * SPAN + oy_) * SPAN + oz_] : nullptr;
                    int tid = -1;
                    if (slot) {
                        tid = *slot;
                    } else {
                        auto it = tid_of.find(cell_key(ox_, oy_, oz_));
                        if (it != tid_of.end()) tid = it->second;
                    }
                    if (tid < 0) {
                        tid = (int)(L.rab.size() / 3);
                        if (tid >= 316) {
                            c->err = "more than 316 distinct translation vectors on a level";
                            return MLF_E_TABLE;
                        }
                        if (slot) *slot = tid;
                        else tid_of.emplace(cell_key(ox_, oy_, oz_), tid);
                        L.rab.insert(L.rab.end(), rh, rh + 3);
                    }
                    L.far_src.push_back(j);
                    L.far_tid.push_back(tid);
                } else if (n == nl) {
                    c->nbox_list.push_back(j);
                }
            }
            L.far_ptr.push_back((int)L.far_src.size());
            if (n == nl) c->nbox_ptr.push_back((int)c->nbox_list.size());
        }
        L.ntrans = (int)(L.rab.size() / 3);
    }
    // near bases of each leaf box: its near boxes' bases, ascending (boxes
    // are independent: sized by a prefix sum, then filled and sorted in parallel)
    {
        const int nbl = c->lv[nl].nb;
        c->near_ptr.assign(nbl + 1, 0);
        for (int i = 0; i < nbl; ++i) {
            long long cnt = 0;
            for (int e = c->nbox_ptr[i]; e < c->nbox_ptr[i + 1]; ++e) {
                const int j = c->nbox_list[e];
                cnt += c->box_ptr[j + 1] - c->box_ptr[j];
            }
            if (c->near_ptr[i] + cnt > 2000000000LL) {
                c->err = "near lists larger than 2^31 entries";
                return MLF_E_ARG;
            }
            c->near_ptr[i + 1] = c->near_ptr[i] + (int)cnt;
        }
        c->near_bases.resize(c->near_ptr[nbl]);
        parallel_for(nbl, [&](int i) {
            int* out = c->near_bases.data() + c->near_ptr[i];
            for (int e = c->nbox_ptr[i]; e < c->nbox_ptr[i + 1]; ++e) {
                const int j = c->nbox_list[e];
                out = std::copy(c->box_bases.begin() + c->box_ptr[j], c->box_bases.begin() + c->box_ptr[j + 1], out);
            }
            std::sort(c->near_bases.begin() + c->near_ptr[i], c->near_bases.begin() + c->near_ptr[i + 1]);
        });
    }
    // near CSR rows in basis order (llenarZesparcida, modMLFMA.f90:1594-1634)
    // the CSR row pointers are int32 (the reference's integer(4) ia_MLFMA)
    long long total = 0;
    for (int m = 0; m < N; ++m) total += c->near_ptr[c->box_of[m] + 1] - c->near_ptr[c->box_of[m]];
    if (total > 2000000000LL) {
        c->err = "near field larger than 2^31 entries";
        return MLF_E_ARG;
    }
    c->ia.assign(N + 1, 0);
    for (int m = 0; m < N; ++m) {
        const int b = c->box_of[m];
        c->ia[m + 1] = c->ia[m] + (c->near_ptr[b + 1] - c->near_ptr[b]);
    }
    c->nnz = c->ia[N];
    c->ja.resize(c->nnz);
    parallel_for(N, [&](int m) {
        const int b = c->box_of[m];
        std::copy(c->near_bases.begin() + c->near_ptr[b], c->near_bases.begin() + c->near_ptr[b + 1],
                  c->ja.begin() + c->ia[m]);
    });
    // interpolation tables and their transposes
    for (int n = 3; n < nl; ++n) {
        Level& L = c->lv[n];
        const Level& Lf = c->lv[n + 1];
        interp_table(L, Lf, L.iw, L.iidx);
        separable_tables(L, Lf, L);
        L.ant_ptr.assign(Lf.K + 1, 0);
        for (int e = 0; e < 9 * L.K; ++e) L.ant_ptr[L.iidx[e] + 1]++;
        for (int q = 0; q < Lf.K; ++q) L.ant_ptr[q + 1] += L.ant_ptr[q];
        L.ant_row.resize(9 * (size_t)L.K);
        L.ant_w.resize(9 * (size_t)L.K);
        std::vector<int> fill(L.ant_ptr.begin(), L.ant_ptr.end() - 1);
        for (int e = 0; e < 9 * L.K; ++e) {   // (row, tap) ascending: the scatter order of Anterpolar
            const int q = L.iidx[e];
            L.ant_row[fill[q]] = e / 9;
            L.ant_w[fill[q]] = L.iw[e];
            fill[q]++;
        }
    }
    return MLF_OK;
}

// Single-level FMM (inicializar_FMM, geomFMM, buscarFuncBases,
// llenar_functransf: modFMM.f90:170-268, 278-469, 650-778) as a one-level
// tree: level 3 is the FMM grid and nlev = 3, so the patterns, translation
// tables, near field and matvec stages are the MLFMA ones without
// interpolation (the receive reads B when nlev = 3).  Box side criterion
// ladomax * lambda (the reference's criterio_ladoW is lambda / 2); the cube of
// side max-extent + lambda/1e4 is cut into ceiling(extent / criterion) boxes
// per axis.  Boxes are visited z-major, then y, then x from the corner
// (max + lambda/2e4) downwards, offsets accumulated by repeated addition, and
// a basis belongs to the first box whose closed bounds hold its edge centre:
// only the (up to 27) grid cells around it can, so each basis tests those in
// visiting order.  Far pairs: |c_i - c_j| >= 2 side - lambda/100, translation
// vectors numbered in order of first appearance (keyed by their grid
// offsets).  Near rows are the near boxes' bases sorted ascending.
int build_fmm(Ctx* c) {
    const int N = c->N;
    const double lambda = c->ph.lambda;
    int lim[6] = {0, 0, 0, 0, 0, 0};
    const double* ec = c->e_centro.data();
    for (int i = 1; i < N; ++i) {
        const double* p = ec + 3 * i;
        if (p[0] > ec[3 * lim[0]]) lim[0] = i;
        if (p[0] < ec[3 * lim[1]]) lim[1] = i;
        if (p[1] > ec[3 * lim[2] + 1]) lim[2] = i;
        if (p[1] < ec[3 * lim[3] + 1]) lim[3] = i;
        if (p[2] > ec[3 * lim[4] + 2]) lim[4] = i;
        if (p[2] < ec[3 * lim[5] + 2]) lim[5] = i;
    }
    const double maxX = ec[3 * lim[0]], minX = ec[3 * lim[1]];
    const double maxY = ec[3 * lim[2] + 1], minY = ec[3 * lim[3] + 1];
    const double maxZ = ec[3 * lim[4] + 2], minZ = ec[3 * lim[5] + 2];
    const double dX = maxX - minX, dY = maxY - minY, dZ = maxZ - minZ;
    double mayor;
    if (dX >= dY && dX >= dZ) mayor = dX;
    else if (dY >= dX && dY >= dZ) mayor = dY;
    else mayor = dZ;
    double tol = lambda / 10000.;
    mayor = mayor + tol;
    tol = tol / 2.;
    const double corner[3] = {maxX + tol, maxY + tol, maxZ + tol};
    const int ne = (int)std::ceil(mayor / (c->ladomax * lambda));
    if (ne < 1 || ne > 400) {
        c->err = "FMM grid of more than 400 boxes per axis";
        return MLF_E_ARG;
    }
    const double lado = mayor / ne;
    c->nlev = 3;
    c->root_side = mayor;
    for (int d = 0; d < 3; ++d) c->root_centre[d] = corner[d] - mayor / 2.;
    Level& L = c->lv[3];
    L.side = lado;
    const double s3 = (double)std::sqrt(3.0f), third = (double)(1.0f / 3.0f);
    const double kd = (2. * PI / lambda) * (s3 * lado);
    L.L = (int)std::floor(kd + 6 * std::pow(kd, third));
    L.nth = L.L;
    L.nph = 2 * L.L;
    L.K = L.nth * L.nph;
    sampling(L);
    // offsets by repeated addition, as the reference's loops accumulate them
    std::vector<double> off(ne);
    {
        double acc = 0.;
        for (int q = 0; q < ne; ++q) { off[q] = acc; acc = acc + lado; }
    }
    auto centre_of = [&](int i, int j, int k, double* cen) {
        cen[0] = (corner[0] - off[k]) - lado / 2.;
        cen[1] = (corner[1] - off[j]) - lado / 2.;
        cen[2] = (corner[2] - off[i]) - lado / 2.;
    };
    // owner cell (loop index i*ne*ne + j*ne + k) of each basis
    std::vector<long long> owner(N, -1);
    for (int n = 0; n < N; ++n) {
        const double* e = ec + 3 * n;
        const int k0 = (int)std::floor((corner[0] - e[0]) / lado);
        const int j0 = (int)std::floor((corner[1] - e[1]) / lado);
        const int i0 = (int)std::floor((corner[2] - e[2]) / lado);
        long long best = -1;
        for (int i = std::max(0, i0 - 1); i <= std::min(ne - 1, i0 + 1); ++i)
            for (int j = std::max(0, j0 - 1); j <= std::min(ne - 1, j0 + 1); ++j)
                for (int k = std::max(0, k0 - 1); k <= std::min(ne - 1, k0 + 1); ++k) {
                    double cen[3];
                    centre_of(i, j, k, cen);
                    const double lq = lado / 2.;
                    if (e[0] <= cen[0] + lq && e[0] >= cen[0] - lq && e[1] <= cen[1] + lq && e[1] >= cen[1] - lq &&
                        e[2] <= cen[2] + lq && e[2] >= cen[2] - lq) {
                        const long long idx = ((long long)i * ne + j) * ne + k;
                        if (best < 0 || idx < best) best = idx;
                    }
                }
        if (best < 0) {
            c->err = "an edge centre lies in no FMM box";
            return MLF_E_STATE;
        }
        owner[n] = best;
    }
    std::vector<int> order(N);
    for (int n = 0; n < N; ++n) order[n] = n;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return owner[a] < owner[b]; });
    c->box_bases.clear();
    c->box_ptr.assign(1, 0);
    L.centre.clear();
    std::vector<int> cell(0);
    for (int t = 0; t < N; ++t) {
        const int n = order[t];
        if (t == 0 || owner[n] != owner[order[t - 1]]) {
            if (t) c->box_ptr.push_back(t);
            const long long idx = owner[n];
            const int i = (int)(idx / ((long long)ne * ne)), j = (int)((idx / ne) % ne), k = (int)(idx % ne);
            double cen[3];
            centre_of(i, j, k, cen);
            L.centre.insert(L.centre.end(), cen, cen + 3);
            cell.push_back(i); cell.push_back(j); cell.push_back(k);
        }
        c->box_bases.push_back(n);
    }
    c->box_ptr.push_back(N);
    L.nb = (int)c->box_ptr.size() - 1;
    L.parent.assign(L.nb, -1);
    L.octant.assign(L.nb, 0);
    c->lv[1].nb = 0;
    c->lv[2].nb = 0;
    c->box_of.assign(N, -1);
    for (int b = 0; b < L.nb; ++b)
        for (int t = c->box_ptr[b]; t < c->box_ptr[b + 1]; ++t) c->box_of[c->box_bases[t]] = b;
    // far / near lists
    const double ftol = lambda / 100.;
    const int span = 2 * ne - 1;
    std::unordered_map<long long, int> tid_of;
    L.far_ptr.assign(1, 0);
    L.far_src.clear();
    L.far_tid.clear();
    L.rab.clear();
    c->near_ptr.assign(1, 0);
    c->near_bases.clear();
    c->nbox_ptr.assign(1, 0);
    c->nbox_list.clear();
    for (int i = 0; i < L.nb; ++i) {
        const size_t near_start = c->near_bases.size();
        for (int j = 0; j < L.nb; ++j) {
            double rh[3];
            for (int d = 0; d < 3; ++d) rh[d] = L.centre[3 * i + d] - L.centre[3 * j + d];
            const double nh = std::sqrt(rh[0] * rh[0] + rh[1] * rh[1] + rh[2] * rh[2]);
            if (nh >= 2 * lado - ftol) {
                // grid offsets (the reference's lambda/100 dedup identifies the same vectors)
                const long long key = ((long long)(cell[3 * j] - cell[3 * i] + ne - 1) * span +
                                       (cell[3 * j + 1] - cell[3 * i + 1] + ne - 1)) * span +
                                      (cell[3 * j + 2] - cell[3 * i + 2] + ne - 1);
                auto it = tid_of.find(key);
                int tid;
                if (it == tid_of.end()) {
                    tid = (int)(L.rab.size() / 3);
                    tid_of.emplace(key, tid);
                    L.rab.insert(L.rab.end(), rh, rh + 3);
                } else {
                    tid = it->second;
                }
                L.far_src.push_back(j);
                L.far_tid.push_back(tid);
            } else {
                c->nbox_list.push_back(j);
                c->near_bases.insert(c->near_bases.end(), c->box_bases.begin() + c->box_ptr[j],
                                     c->box_bases.begin() + c->box_ptr[j + 1]);
            }
        }
        L.far_ptr.push_back((int)L.far_src.size());
        std::sort(c->near_bases.begin() + near_start, c->near_bases.end());
        c->near_ptr.push_back((int)c->near_bases.size());
        c->nbox_ptr.push_back((int)c->nbox_list.size());
    }
    L.ntrans = (int)(L.rab.size() / 3);
    // the CSR row pointers are int32 (the reference's integer(4) ia_MLFMA)
    long long total = 0;
    for (int m = 0; m < N; ++m) total += c->near_ptr[c->box_of[m] + 1] - c->near_ptr[c->box_of[m]];
    if (total > 2000000000LL) {
        c->err = "near field larger than 2^31 entries";
        return MLF_E_ARG;
    }
    c->ia.assign(N + 1, 0);
    for (int m = 0; m < N; ++m) {
        const int b = c->box_of[m];
        c->ia[m + 1] = c->ia[m] + (c->near_ptr[b + 1] - c->near_ptr[b]);
    }
    c->nnz = c->ia[N];
    c->ja.resize(c->nnz);
    parallel_for(N, [&](int m) {
        const int b = c->box_of[m];
        std::copy(c->near_bases.begin() + c->near_ptr[b], c->near_bases.begin() + c->near_ptr[b + 1],
                  c->ja.begin() + c->ia[m]);
    });
    return MLF_OK;
}

// ---------------------------------------------------------------------------
// ILU(0)
// ---------------------------------------------------------------------------

namespace {
inline float2 mulf(float2 a, float2 b) {
    // complex(4) * complex(4) in single precision
    const float p1 = a.x * b.x, p2 = a.y * b.y, p3 = a.x * b.y, p4 = a.y * b.x;
    return make_float2(p1 - p2, p3 + p4);
}
}  // namespace

// ilu0C, modIterativo.f90:1805-1976: Saad's ILU(0) (SPARSKIT ilu0), IKJ on the
// CSR pattern, restated step by step because the tests hold the complex(4)
// factors bit-exact against the reference's.  MSR output with 1-based
// content: alu[1..n] inverted diagonal, jlu[1] = n+2, row i of L then U in
// [jlu[i], jlu[i+1]), ju[i] = start of U.  Factors are complex(4); the update
// alu(jw) - tl*alu(jj) runs in double, tl = alu(j) * alu(jrow) in single, as
// in the reference.  A row without a diagonal entry keeps alu[i] = 0 and is
// reported as that zero pivot.  Returns 0 or the zero-pivot row.
int ilu0_msr(int n, const int* ia, const int* ja, const float2* zf, float2* alu, int* jlu, int* ju) {
    std::vector<int> iw(n + 1, 0);
    long long ju0 = n + 2;
    jlu[1] = (int)ju0;
    for (int ii = 1; ii <= n; ++ii) {
        const long long js = ju0;
        for (long long j = ia[ii - 1]; j < ia[ii]; ++j) {
            const int jcol = ja[j] + 1;
            if (jcol == ii) {
                alu[ii] = zf[j];
                iw[jcol] = ii;
                ju[ii] = (int)ju0;
            } else {
                alu[ju0] = zf[j];
                jlu[ju0] = jcol;
                iw[jcol] = (int)ju0;
                ++ju0;
            }
        }
        jlu[ii + 1] = (int)ju0;
        const long long jf = ju0 - 1;
        const long long jm = ju[ii] - 1;
        for (long long j = js; j <= jm; ++j) {
            const int jrow = jlu[j];
            const float2 tlf = mulf(alu[j], alu[jrow]);
            alu[j] = tlf;
            const double tr = tlf.x, ti = tlf.y;
            for (long long jj = ju[jrow]; jj < jlu[jrow + 1]; ++jj) {
                const int jw = iw[jlu[jj]];
                if (jw != 0) {
                    const double ar = alu[jj].x, ai = alu[jj].y;
                    const double rr = (double)alu[jw].x - (tr * ar - ti * ai);
                    const double ri = (double)alu[jw].y - (tr * ai + ti * ar);
                    alu[jw] = make_float2((float)rr, (float)ri);
                }
            }
        }
        if (alu[ii].x == 0.0f && alu[ii].y == 0.0f) return ii;
        const double dr = alu[ii].x, di = alu[ii].y, den = dr * dr + di * di;
        alu[ii] = make_float2((float)(dr / den), (float)(-di / den));
        iw[ii] = 0;
        for (long long i = js; i <= jf; ++i) iw[jlu[i]] = 0;
    }
    return 0;
}

// ILU(0) of the context's near field (crear_precond ILU0 branch,
// main.f90:851-902): the device values are fetched and factorised on the host
// as the reference does.  Returns 0, the zero-pivot row, or -1 on a CUDA error.
int ilu0_factor(Ctx* c) {
    const int n = c->N;
    const long long nnz = c->nnz;
    c->alu.assign(nnz + 2, make_float2(0.f, 0.f));
    c->jlu.assign(nnz + 2, 0);
    c->ju.assign(n + 1, 0);
    std::vector<float2> zf;
    if (fetch_near_values(c, zf) != MLF_OK) return -1;
    return ilu0_msr(n, c->ia.data(), c->ja.data(), zf.data(), c->alu.data(), c->jlu.data(), c->ju.data());
}

// ilutC, modIterativo.f90:2432-2883 (Saad's dual-threshold ILUT as adapted
// to complex in the reference) with bsort2C (:1673-1748).  Row ii: entries
// with |a| >= tol*tnorm (tnorm = mean |a| of the row) are unpacked into an L
// and a U work row; rows jrow < ii are eliminated in increasing column order,
// a multiplier fact = wl*alu(jrow) is dropped when |fact| * unorm(jrow) <=
// tol*tnorm, small fill-ins are dropped; then the len = min(nl, lenl0+lfil)
// largest multipliers (bubble-sorted by modulus) form the L row and the
// diagonal plus the len-1 largest of the rest form the U row; unorm(ii) =
// sum |U offdiag kept| / (len+1).  Factors are complex(4) (rounded on store),
// work rows complex(8).  When the diagonal is not the first U entry the
// reference swaps with a stale index (wu(j) = wu(idiag)); this restatement
// swaps into position 1, the evident intent.  Returns ierr as the reference:
// 0, the zero-pivot row, or -5 for a zero U diagonal.
int ilut_factor(Ctx* c, int lfil, double tol) {
    const int n = c->N;
    std::vector<float2> zf;
    if (fetch_near_values(c, zf) != MLF_OK) return -100;
    std::vector<float2> alu(n + 2);
    std::vector<int> jlu(n + 2), ju(n + 1, 0);
    std::vector<int> jr(n + 1, 0), jwl(n + 1), jwu(n + 1);
    std::vector<double> wlr(n + 2), wli(n + 2), wur(n + 2), wui(n + 2), unorm(n + 2, 0.0);
    long long ju0 = n + 2;
    jlu[1] = (int)ju0;
    auto cab = [](double r, double i) { return std::hypot(r, i); };
    auto bsort = [&](double* wr, double* wi, int* ind, int nn, int ncut) {
        int i = 1;
        for (;;) {
            bool test = false;
            for (int j = nn - 1; j >= i; --j) {
                if (cab(wr[j - 1], wi[j - 1]) < cab(wr[j], wi[j])) {
                    std::swap(wr[j - 1], wr[j]);
                    std::swap(wi[j - 1], wi[j]);
                    std::swap(ind[j - 1], ind[j]);
                    test = true;
                }
            }
            ++i;
            if (!test || ncut < i) break;
        }
    };
    for (int ii = 1; ii <= n; ++ii) {
        const long long j1 = c->ia[ii - 1], j2 = c->ia[ii] - 1;
        int lenu = 0, lenl = 0;
        double tnorm = 0.0;
        for (long long k = j1; k <= j2; ++k) tnorm = tnorm + cab(zf[k].x, zf[k].y);
        tnorm = tnorm / (double)(j2 - j1 + 1);
        for (long long j = j1; j <= j2; ++j) {
            const int k = c->ja[j] + 1;
            const double tr = zf[j].x, ti = zf[j].y;
            if (tol * tnorm <= cab(tr, ti)) {
                if (k < ii) {
                    ++lenl; jwl[lenl] = k; wlr[lenl] = tr; wli[lenl] = ti; jr[k] = lenl;
                } else {
                    ++lenu; jwu[lenu] = k; wur[lenu] = tr; wui[lenu] = ti; jr[k] = lenu;
                }
            }
        }
        const int lenl0 = lenl, lenu0 = lenu;
        int jjj = 0, nl = 0;
        for (;;) {
            ++jjj;
            if (lenl < jjj) break;
            int jrow = jwl[jjj], kk = jjj;
            for (int j = jjj + 1; j <= lenl; ++j)
                if (jwl[j] < jrow) { jrow = jwl[j]; kk = j; }
            const int jold = jwl[jjj];
            jwl[jjj] = jrow; jwl[kk] = jold;
            jr[jrow] = jjj; jr[jold] = kk;
            std::swap(wlr[kk], wlr[jjj]);
            std::swap(wli[kk], wli[jjj]);
            if (ii <= jrow) break;
            // fact = wl(jjj) * alu(jrow): complex(8) x complex(4)
            const double ar = alu[jrow].x, ai = alu[jrow].y;
            const double fr = wlr[jjj] * ar - wli[jjj] * ai, fi = wlr[jjj] * ai + wli[jjj] * ar;
            jr[jrow] = 0;
            if (cab(fr, fi) * unorm[jrow] <= tol * tnorm) continue;
            for (int k = ju[jrow]; k < jlu[jrow + 1]; ++k) {
                const double sr = fr * alu[k].x - fi * alu[k].y, si = fr * alu[k].y + fi * alu[k].x;
                const int j = jlu[k];
                const int jpos = jr[j];
                if (cab(sr, si) < tol * tnorm && jpos == 0) continue;
                if (ii <= j) {
                    if (jpos == 0) {
                        ++lenu;
                        if (n < lenu) return -1;
                        jwu[lenu] = j; jr[j] = lenu; wur[lenu] = -sr; wui[lenu] = -si;
                    } else {
                        wur[jpos] = wur[jpos] - sr; wui[jpos] = wui[jpos] - si;
                    }
                } else {
                    if (jpos == 0) {
                        ++lenl;
                        if (n < lenl) return -1;
                        jwl[lenl] = j; jr[j] = lenl; wlr[lenl] = -sr; wli[lenl] = -si;
                    } else {
                        wlr[jpos] = wlr[jpos] - sr; wli[jpos] = wli[jpos] - si;
                    }
                }
            }
            ++nl;
            wlr[nl] = fr; wli[nl] = fi; jwl[nl] = jrow;
        }
        int len = std::min(nl, lenl0 + lfil);
        bsort(&wlr[1], &wli[1], &jwl[1], nl, len);
        for (int k = 1; k <= len; ++k) {
            alu.push_back(make_float2((float)wlr[k], (float)wli[k]));
            jlu.push_back(jwl[k]);
            ++ju0;
        }
        ju[ii] = (int)ju0;
        for (int k = jjj; k <= lenl; ++k) jr[jwl[k]] = 0;
        const int idiag = jr[ii];
        if (idiag == 0) return ii;
        if (idiag != 1) {
            std::swap(wur[1], wur[idiag]);
            std::swap(wui[1], wui[idiag]);
            std::swap(jwu[1], jwu[idiag]);
        }
        len = std::min(lenu, lenu0 + lfil);
        bsort(&wur[2], &wui[2], &jwu[2], lenu - 1, len);
        double t = 0.0;
        for (int k = 2; k <= len; ++k) {
            jlu.push_back(jwu[k]);
            alu.push_back(make_float2((float)wur[k], (float)wui[k]));
            t = t + cab(wur[k], wui[k]);
            ++ju0;
        }
        unorm[ii] = t / (double)(len + 1);
        if (cab(wur[1], wui[1]) == 0.0) return -5;
        const double dr = wur[1], di = wui[1], den = dr * dr + di * di;
        alu[ii] = make_float2((float)(dr / den), (float)(-di / den));
        jlu[ii + 1] = (int)ju0;
        for (int k = 1; k <= lenu; ++k) jr[jwu[k]] = 0;
    }
    c->alu.swap(alu);
    c->jlu.swap(jlu);
    c->ju.swap(ju);
    c->alu.push_back(make_float2(0, 0));
    c->jlu.push_back(0);
    return 0;
}

// Level schedules: forward row i waits on the L columns of row i, backward
// row i on its U columns.  Rows of one level are independent.
void ilu_levels(Ctx* c) {
    const int n = c->N;
    std::vector<int> lev(n + 1, 0);
    int maxl = 0;
    for (int i = 1; i <= n; ++i) {
        int l = 0;
        for (int k = c->jlu[i]; k < c->ju[i]; ++k) l = std::max(l, lev[c->jlu[k]] + 1);
        lev[i] = l;
        maxl = std::max(maxl, l);
    }
    c->lvl_ptr_f.assign(maxl + 2, 0);
    for (int i = 1; i <= n; ++i) c->lvl_ptr_f[lev[i] + 1]++;
    for (int l = 0; l <= maxl; ++l) c->lvl_ptr_f[l + 1] += c->lvl_ptr_f[l];
    c->lvl_rows_f.assign(n, 0);
    {
        std::vector<int> f(c->lvl_ptr_f.begin(), c->lvl_ptr_f.end() - 1);
        for (int i = 1; i <= n; ++i) c->lvl_rows_f[f[lev[i]]++] = i;
    }
    std::fill(lev.begin(), lev.end(), 0);
    maxl = 0;
    for (int i = n; i >= 1; --i) {
        int l = 0;
        for (int k = c->ju[i]; k < c->jlu[i + 1]; ++k) l = std::max(l, lev[c->jlu[k]] + 1);
        lev[i] = l;
        maxl = std::max(maxl, l);
    }
    c->lvl_ptr_b.assign(maxl + 2, 0);
    for (int i = 1; i <= n; ++i) c->lvl_ptr_b[lev[i] + 1]++;
    for (int l = 0; l <= maxl; ++l) c->lvl_ptr_b[l + 1] += c->lvl_ptr_b[l];
    c->lvl_rows_b.assign(n, 0);
    {
        std::vector<int> f(c->lvl_ptr_b.begin(), c->lvl_ptr_b.end() - 1);
        for (int i = n; i >= 1; --i) c->lvl_rows_b[f[lev[i]]++] = i;
    }
}

}  // namespace mlf
