/*
 * ORACLE — test infrastructure only.  A plain-C restatement of MLFMAxwell's
 * iterative solve (the reference is serial Fortran 90), used by tests/, by
 * __graft_entry__.smoke() and by bench.py's cpu_baseline / reference arm as
 * the checker and as the CPU baseline.  Nothing in the lywell_gb300 product
 * path links, loads or calls this file.
 *
 * Parity is pinned against the reference's own outputs: golden fixtures made
 * by running the reference's shipped binary on synthetic meshes, and the
 * reference's committed known-answer files (ILU0 10x10, interpolation dump);
 * see tests/golden/make_golden.py.
 *
 * Every function cites the reference routine it restates (file:line, paths
 * inside the reference project).  The arithmetic order of the reference is
 * kept where it is observable: single-precision literals such as (1./3.),
 * sqrt(3.), log10(2.), (1./72.) are evaluated in float and promoted, the
 * near-field matrix is stored as complex(4) (float pairs), the ILU0 factors
 * are complex(4) with the reference's mixed float/double updates.
 *
 * Build: oracle/Makefile (gcc -O2 -ffp-contract=off -fopenmp).
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;
typedef float complex cplxf;

/* modGlobalParam.f90:12-17 */
static const double PI = 3.141592653589793;
static const double MU = 1.2566370614E-6;
static const double EPSI = 8.8541878176E-12;

typedef struct {
    double lambda, w, kappa, vp, smue; /* smue = sqrt(mu*epsi) */
} Phys;

/* setlambda, modGlobalParam.f90:52-61 */
static Phys phys_from_lambda(double lambda) {
    Phys p;
    p.vp = 1.0 / sqrt(MU * EPSI);
    p.lambda = lambda;
    p.w = 2. * PI * p.vp / lambda;
    p.kappa = 2. * PI / lambda;
    p.smue = sqrt(MU * EPSI);
    return p;
}

/* ------------------------------------------------------------------ */
/* special functions                                                    */
/* ------------------------------------------------------------------ */

/* factorial, modGlobalMetod.f90:1004-1015: sequential product in double */
static double factorial(int x) {
    double r = 1.;
    for (int i = 1; i <= x; i++) r = r * i;
    return r;
}

/* legendre, modGlobalMetod.f90:988-1002: explicit binomial-square sum
 *   P_n(x) = 0.5^n * sum_i (n!/(i!(n-i)!))^2 (x+1)^(n-i) (x-1)^i
 * Powers are formed by repeated multiplication, left to right.
 * mode 1 evaluates P_n by the three-term (Bonnet) recurrence instead. */
static void legendre_all(int nmax, double x, int mode, double* P) {
    if (mode == 1) {
        P[0] = 1.0;
        if (nmax >= 1) P[1] = x;
        for (int n = 1; n < nmax; n++)
            P[n + 1] = ((2.0 * n + 1.0) * x * P[n] - n * P[n - 1]) / (n + 1.0);
        return;
    }
    double pa[512], pb[512];
    double a = x + 1, b = x - 1;
    pa[0] = 1.0; pb[0] = 1.0;
    for (int k = 1; k <= nmax; k++) { pa[k] = pa[k - 1] * a; pb[k] = pb[k - 1] * b; }
    for (int n = 0; n <= nmax; n++) {
        double fn = factorial(n);
        double r = 0.;
        for (int i = 0; i <= n; i++) {
            double c = fn / (factorial(i) * factorial(n - i));
            r = r + (c * c) * pa[n - i] * pb[i];
        }
        P[n] = ldexp(1.0, -n) * r;   /* (0.5**n) is exact */
    }
}

/* Spherical Bessel functions j_n, y_n for n = 0..nmax at x > 0.
 * y_n: upward three-term recurrence (stable for all n).  j_n: upward
 * recurrence when nmax <= x (the only case the translation operator needs,
 * since its series stops at floor(kD)), otherwise Miller's downward
 * recurrence from well above max(nmax, x), normalised by j_0 or j_1.
 * These stand in for the Zhang-Jin routines sphj/sphy
 * (modGlobalMetod.f90:777-979) used through hankel (modGlobalMetod.f90:493-502). */
static void sph_bessel(int nmax, double x, double* j, double* y) {
    double s = sin(x), c = cos(x);
    y[0] = -c / x;
    if (nmax >= 1) y[1] = -c / (x * x) - s / x;
    for (int n = 1; n < nmax; n++) y[n + 1] = (2.0 * n + 1.0) / x * y[n] - y[n - 1];
    double j0 = s / x, j1 = s / (x * x) - c / x;
    if ((double)nmax <= x) {
        j[0] = j0;
        if (nmax >= 1) j[1] = j1;
        for (int n = 1; n < nmax; n++) j[n + 1] = (2.0 * n + 1.0) / x * j[n] - j[n - 1];
        return;
    }
    int top = (nmax > (int)x ? nmax : (int)x) + 30 + (int)(10.0 * cbrt(x + 1.0));
    double fp1 = 0.0, f = 1e-280;
    for (int n = top; n >= 1; n--) {
        double fm1 = (2.0 * n + 1.0) / x * f - fp1;
        fp1 = f;
        f = fm1;
        if (n - 1 <= nmax) j[n - 1] = f;
        if (fabs(f) > 1e250) {
            f *= 1e-250;
            fp1 *= 1e-250;
            for (int q = n - 1; q <= nmax; q++) if (q >= 0) j[q] *= 1e-250;
        }
    }
    double scale = fabs(j0) > fabs(j1) ? j0 / j[0] : j1 / j[1];
    for (int n = 0; n <= nmax; n++) j[n] *= scale;
}

/* exposed for the special-function tests */
void ora_sph_bessel(int nmax, double x, double* j, double* y) { sph_bessel(nmax, x, j, y); }
void ora_legendre(int nmax, double x, int mode, double* P) { legendre_all(nmax, x, mode, P); }

/* ------------------------------------------------------------------ */
/* context                                                              */
/* ------------------------------------------------------------------ */

typedef struct {
    int nb;
    double side;
    int L, nth, nph, K;
    double* centre;   /* nb*3 */
    int* parent;      /* nb, 0-based index at level-1 (-1 at level 1) */
    int* child_ptr;   /* nb+1 : children range at level+1 */
    int cap;
    int npadres;
    /* sampling (level >= 3) */
    double *kap, *ath, *aph, *ang, *wq;
    /* translation lists (level >= 3) */
    int* far_ptr;
    int *far_src, *far_tid;
    int ntrans;
    double* rab;       /* ntrans*3 */
    cplx* T;           /* ntrans*K */
    /* interpolation level+1 -> level (3 <= level < nlev) */
    double* iw;
    int* iidx;         /* K*9, 0-based sample index at level+1 */
    cplx *C, *B, *A;   /* nb*2*K */
} Level;

typedef struct {
    Phys ph;
    double ladomax;
    int legendre_mode;
    int N, T, P;
    const double *p_coord, *t_baric, *t_baric_sub, *e_long, *e_centro;
    const int *e_t, *e_po; /* 0-based */
    int nlev;
    Level lv[32];          /* 1-based by level number */
    double root_centre[3], root_side;
    /* leaf boxes */
    int* box_ptr;          /* nb+1 */
    int* box_bases;        /* N */
    int* box_of;           /* N: leaf box of each basis */
    int* near_ptr;         /* nb+1 into near_bases */
    int* near_bases;
    /* patterns funcRAD(K,2,N) as [N][2][K] */
    cplx* frad;
    /* near CSR (0-based), complex(4) */
    int64_t nnz;
    int* ia;               /* N+1 */
    int* ja;               /* nnz */
    cplxf* zn;             /* nnz */
    /* ILU0 factors, MSR layout of ilu0C (1-based content) */
    cplxf* alu;
    int* jlu;
    int* ju;
    int ilu_status;        /* -1 not built */
    cplx* minv;            /* neighbourhood-inverse preconditioner, near CSR pattern */
    int nthreads;
} Ctx;

static void* xcalloc(size_t n, size_t s) { void* p = calloc(n ? n : 1, s); return p; }

/* limites_dispersor, modGlobalMetod.f90:386-434 */
static void limites(const double* ec, int N, int lim[6]) {
    for (int k = 0; k < 6; k++) lim[k] = 0;
    for (int i = 1; i < N; i++) {
        const double* c = ec + 3 * i;
        if (c[0] > ec[3 * lim[0] + 0]) lim[0] = i;
        if (c[0] < ec[3 * lim[1] + 0]) lim[1] = i;
        if (c[1] > ec[3 * lim[2] + 1]) lim[2] = i;
        if (c[1] < ec[3 * lim[3] + 1]) lim[3] = i;
        if (c[2] > ec[3 * lim[4] + 2]) lim[4] = i;
        if (c[2] < ec[3 * lim[5] + 2]) lim[5] = i;
    }
}

static void lv_append(Level* L, const double c[3], int parent) {
    if (L->nb == L->cap) {
        L->cap = L->cap ? 2 * L->cap : 64;
        L->centre = realloc(L->centre, sizeof(double) * 3 * L->cap);
        L->parent = realloc(L->parent, sizeof(int) * L->cap);
    }
    memcpy(L->centre + 3 * L->nb, c, 3 * sizeof(double));
    L->parent[L->nb] = parent;
    L->nb++;
}

typedef struct { int* b; int n, cap; } IVec;
static void iv_push(IVec* v, int x) {
    if (v->n == v->cap) { v->cap = v->cap ? 2 * v->cap : 1024; v->b = realloc(v->b, sizeof(int) * v->cap); }
    v->b[v->n++] = x;
}

/* geomMLFMA, dividir_en_8_hijos, buscarFuncBases: modMLFMA.f90:497-581, 706-833 */
static void geom(Ctx* c, const double centro[3], double lcubo, const int* vb, int nvb, int nivel,
                 IVec* leaf_bases, IVec* leaf_ptr) {
    if (nivel == c->nlev) return;
    double lh = lcubo / 2., lq = lcubo / 4.;
    static const int sx[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
    static const int sy[8] = {-1, 1, -1, 1, -1, 1, -1, 1};
    static const int sz[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
    int* work = malloc(sizeof(int) * (nvb ? nvb : 1));
    int* found = malloc(sizeof(int) * (nvb ? nvb : 1));
    int* rest = malloc(sizeof(int) * (nvb ? nvb : 1));
    memcpy(work, vb, sizeof(int) * nvb);
    int nw = nvb;
    Level* child = &c->lv[nivel + 1];
    child->npadres++;
    int padre = child->npadres - 1;
    for (int i = 0; i < 8; i++) {
        double ch[3];
        ch[0] = sx[i] < 0 ? centro[0] - lq : centro[0] + lq;
        ch[1] = sy[i] < 0 ? centro[1] - lq : centro[1] + lq;
        ch[2] = sz[i] < 0 ? centro[2] - lq : centro[2] + lq;
        double q = lh / 2.;
        double xmax = ch[0] + q, xmin = ch[0] - q, ymax = ch[1] + q, ymin = ch[1] - q;
        double zmax = ch[2] + q, zmin = ch[2] - q;
        int nf = 0, nr = 0;
        for (int t = 0; t < nw; t++) {
            const double* e = c->e_centro + 3 * work[t];
            if (e[0] <= xmax && e[0] >= xmin && e[1] <= ymax && e[1] >= ymin && e[2] <= zmax && e[2] >= zmin)
                found[nf++] = work[t];
            else
                rest[nr++] = work[t];
        }
        if (nf > 0) {
            lv_append(child, ch, padre);
            if (nivel + 1 == c->nlev) {
                for (int t = 0; t < nf; t++) iv_push(leaf_bases, found[t]);
                iv_push(leaf_ptr, leaf_bases->n);
            }
            geom(c, ch, lh, found, nf, nivel + 1, leaf_bases, leaf_ptr);
            memcpy(work, rest, sizeof(int) * nr);
            nw = nr;
        }
    }
    free(work); free(found); free(rest);
}

/* llenar_kappas, modMLFMA.f90:453-495 */
static void fill_kappas(Level* L) {
    int K = L->K;
    L->kap = malloc(sizeof(double) * 3 * K); L->ath = malloc(sizeof(double) * 3 * K);
    L->aph = malloc(sizeof(double) * 3 * K); L->ang = malloc(sizeof(double) * 2 * K);
    L->wq = malloc(sizeof(double) * K);
    double dphi = 2. * PI / L->nph, dth = PI / L->nth;
    int cont = 0;
    for (int j = 1; j <= L->nph; j++) {
        double phi = (dphi / 2.) * ((2 * j) - 1);
        for (int k = 1; k <= L->nth; k++) {
            double th = (dth / 2.) * ((2 * k) - 1);
            double st = sin(th), ct = cos(th), sp = sin(phi), cp = cos(phi);
            L->kap[3 * cont + 0] = st * cp; L->kap[3 * cont + 1] = st * sp; L->kap[3 * cont + 2] = ct;
            L->ath[3 * cont + 0] = ct * cp; L->ath[3 * cont + 1] = ct * sp; L->ath[3 * cont + 2] = -st;
            L->aph[3 * cont + 0] = -sp; L->aph[3 * cont + 1] = cp; L->aph[3 * cont + 2] = 0.;
            L->ang[2 * cont + 0] = th; L->ang[2 * cont + 1] = phi;
            L->wq[cont] = (cos((k - 1) * dth) - cos(k * dth)) * dphi;
            cont++;
        }
    }
}

/* calc_functransf, modMLFMA.f90:964-994 */
static void calc_functransf(const Ctx* c, const Level* L, const double rab[3], cplx* v) {
    int Ltrue = L->L;
    double modul = sqrt(rab[0] * rab[0] + rab[1] * rab[1] + rab[2] * rab[2]);
    double kD = (2. * PI / c->ph.lambda) * modul;
    int kDint = (int)kD;
    if (kDint < Ltrue) Ltrue = kDint;
    double jb[512], yb[512], P[512];
    if (Ltrue > 500) Ltrue = 500;
    sph_bessel(Ltrue, kD, jb, yb);
    cplx h[512], cf[512];
    for (int l = 0; l <= Ltrue; l++) {
        h[l] = jb[l] - I * yb[l];     /* hankel = j - jj*y */
        /* ((-jj)**(l+1)) * ((2.*l)+1) */
        int m = (l + 1) & 3;
        double f = 2. * l + 1;
        cplx p = m == 0 ? 1.0 : m == 1 ? -I : m == 2 ? -1.0 : I;
        cf[l] = p * f;
    }
    double u[3] = {rab[0] / modul, rab[1] / modul, rab[2] / modul};
    for (int i = 0; i < L->K; i++) {
        const double* kk = L->kap + 3 * i;
        double x = kk[0] * u[0] + kk[1] * u[1] + kk[2] * u[2];
        legendre_all(Ltrue, x, c->legendre_mode, P);
        double vr = 0., vi = 0.;
        for (int l = 0; l <= Ltrue; l++) {
            /* (cf*h)*P, cf purely real or imaginary */
            double ar = creal(cf[l]), ai = cimag(cf[l]);
            double tr = ar * creal(h[l]) - ai * cimag(h[l]);
            double ti = ar * cimag(h[l]) + ai * creal(h[l]);
            vr = vr + tr * P[l];
            vi = vi + ti * P[l];
        }
        double s = (2. * PI / c->ph.lambda) / (4. * PI);
        v[i] = vr * s + I * (vi * s);
    }
}

/* llenar_functransf, modMLFMA.f90:835-960 (far lists, unique displacements, near lists) */
static int build_lists(Ctx* c) {
    double tol = c->ph.lambda / 100.;
    int nl = c->nlev;
    for (int n = 3; n <= nl; n++) {
        Level* L = &c->lv[n];
        Level* Lp = &c->lv[n - 1];
        L->far_ptr = xcalloc(L->nb + 1, sizeof(int));
        IVec fs = {0}, ft = {0};
        double* rab = xcalloc(3 * 316, sizeof(double));
        int cont = 0;
        IVec nearb = {0}, nearp = {0};
        if (n == nl) iv_push(&nearp, 0);
        for (int i = 0; i < L->nb; i++) {
            int ip = L->parent[i];
            int nstart = nearb.n;
            for (int j = 0; j < L->nb; j++) {
                int jp = L->parent[j];
                double rp[3], rh[3];
                for (int d = 0; d < 3; d++) rp[d] = Lp->centre[3 * ip + d] - Lp->centre[3 * jp + d];
                double np_ = sqrt(rp[0] * rp[0] + rp[1] * rp[1] + rp[2] * rp[2]);
                if (!(np_ < (2 * Lp->side - tol))) continue;
                for (int d = 0; d < 3; d++) rh[d] = L->centre[3 * i + d] - L->centre[3 * j + d];
                double nh = sqrt(rh[0] * rh[0] + rh[1] * rh[1] + rh[2] * rh[2]);
                if (nh >= (2 * L->side - tol)) {
                    int k;
                    for (k = 0; k < cont; k++) {
                        if (fabs(rab[3 * k] - rh[0]) < tol && fabs(rab[3 * k + 1] - rh[1]) < tol &&
                            fabs(rab[3 * k + 2] - rh[2]) < tol)
                            break;
                    }
                    if (k == cont) {
                        if (cont == 316) return -10;
                        memcpy(rab + 3 * cont, rh, sizeof(rh));
                        cont++;
                    }
                    iv_push(&fs, j);
                    iv_push(&ft, k);
                } else if (n == nl) {
                    for (int t = c->box_ptr[j]; t < c->box_ptr[j + 1]; t++) iv_push(&nearb, c->box_bases[t]);
                }
            }
            L->far_ptr[i + 1] = fs.n;
            if (n == nl) {
                /* Sort ascending (Sort, modGlobalMetod.f90:1241-1292) */
                int cnt = nearb.n - nstart;
                int* a = nearb.b + nstart;
                for (int t = 1; t < cnt; t++) {  /* insertion sort, lists are ~100 long */
                    int v = a[t], q = t - 1;
                    while (q >= 0 && a[q] > v) { a[q + 1] = a[q]; q--; }
                    a[q + 1] = v;
                }
                iv_push(&nearp, nearb.n);
            }
        }
        L->far_src = fs.b ? fs.b : xcalloc(1, sizeof(int));
        L->far_tid = ft.b ? ft.b : xcalloc(1, sizeof(int));
        L->ntrans = cont;
        L->rab = rab;
        if (n == nl) {
            c->near_ptr = nearp.b;
            c->near_bases = nearb.b;
        }
    }
    return 0;
}

static void fill_trans(Ctx* c) {
    for (int n = 3; n <= c->nlev; n++) {
        Level* L = &c->lv[n];
        L->T = xcalloc((size_t)L->ntrans * L->K, sizeof(cplx));
#pragma omp parallel for schedule(dynamic)
        for (int t = 0; t < L->ntrans; t++) calc_functransf(c, L, L->rab + 3 * t, L->T + (size_t)t * L->K);
    }
}

/* Wlagrange3, modMLFMA.f90:1318-1341 */
static void wlagrange3(double x, const double xm[3], double W[3]) {
    for (int i = 0; i < 3; i++) {
        double ww = 1.;
        for (int j = 0; j < 3; j++)
            if (j != i) ww = ww * ((x - xm[j]) / (xm[i] - xm[j]));
        W[i] = ww;
    }
}

/* hallarKcercanos, modMLFMA.f90:1096-1315: nearest child sample by binary
 * search in theta and in phi, neighbours with wrap-around at both ends. */
static void hallar_kcercanos(const Level* Lc /*fine*/, double theta, double phi, int V[9]) {
    int nph = Lc->nph, nth = Lc->nth;
    const double* ang = Lc->ang;
    long techo = 1, piso = nph, posmid;
    double del = ang[2 * (nth + 1 - 1) + 1] - ang[2 * 0 + 1];
    for (;;) {
        posmid = (techo + piso) / 2;
        double valorpos = ang[2 * ((posmid - 1) * nth) + 1];
        if (posmid == techo || posmid == piso) {
            if (fabs(phi - ang[2 * ((techo - 1) * nth) + 1]) < fabs(phi - ang[2 * ((piso - 1) * nth) + 1]))
                posmid = techo;
            else
                posmid = piso;
            break;
        }
        if (valorpos == phi) break;
        if (del > 0) {
            if (valorpos > phi) piso = posmid;
            else if (valorpos < phi) techo = posmid;
        } else {
            if (valorpos > phi) techo = posmid;
            else if (valorpos < phi) piso = posmid;
        }
    }
    long posPhi = posmid, posPhimay, posPhimen;
    if (del > 0) {
        if (posPhi == 1) { posPhimay = posPhi + 1; posPhimen = nph; }
        else if (posPhi == nph) { posPhimay = 1; posPhimen = posPhi - 1; }
        else { posPhimen = posPhi - 1; posPhimay = posPhi + 1; }
    } else {
        if (posPhi == 1) { posPhimen = posPhi + 1; posPhimay = nph; }
        else if (posPhi == nph) { posPhimen = 1; posPhimay = posPhi - 1; }
        else { posPhimay = posPhi - 1; posPhimen = posPhi + 1; }
    }
    techo = 1; piso = nth;
    del = ang[2 * 1 + 0] - ang[2 * 0 + 0];
    for (;;) {
        posmid = (techo + piso) / 2;
        double valorpos = ang[2 * (posmid - 1) + 0];
        if (posmid == techo || posmid == piso) {
            if (fabs(theta - ang[2 * (techo - 1) + 0]) < fabs(theta - ang[2 * (piso - 1) + 0]))
                posmid = techo;
            else
                posmid = piso;
            break;
        }
        if (valorpos == theta) break;
        if (del > 0) {
            if (valorpos > theta) piso = posmid;
            else if (valorpos < theta) techo = posmid;
        } else {
            if (valorpos > theta) techo = posmid;
            else if (valorpos < theta) piso = posmid;
        }
    }
    long posT = posmid, posTmay, posTmen;
    if (del > 0) {
        if (posT == 1) { posTmen = nth; posTmay = posT + 1; }
        else if (posT == nth) { posTmen = posT - 1; posTmay = 1; }
        else { posTmay = posT + 1; posTmen = posT - 1; }
    } else {
        if (posT == 1) { posTmay = nth; posTmen = posT + 1; }
        else if (posT == nth) { posTmay = posT - 1; posTmen = 1; }
        else { posTmen = posT + 1; posTmay = posT - 1; }
    }
    long base[3] = {posPhi, posPhimen, posPhimay};
    long th[3] = {posT, posTmen, posTmay};
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) V[3 * a + b] = (int)(nth * (base[a] - 1) + th[b]); /* 1-based */
}

/* llenarMinterp, modMLFMA.f90:998-1092 for one (coarse, fine) pair of grids */
static void build_interp(const Level* Lp, const Level* Lc, double* iw, int* iidx) {
    for (int i = 0; i < Lp->K; i++) {
        double xt = Lp->ang[2 * i], xp = Lp->ang[2 * i + 1];
        int V[9];
        hallar_kcercanos(Lc, xt, xp, V);
        double mt[3] = {Lc->ang[2 * (V[0] - 1)], Lc->ang[2 * (V[1] - 1)], Lc->ang[2 * (V[2] - 1)]};
        double mp[3] = {Lc->ang[2 * (V[0] - 1) + 1], Lc->ang[2 * (V[3] - 1) + 1], Lc->ang[2 * (V[6] - 1) + 1]};
        double Wt[3], Wp[3];
        wlagrange3(xt, mt, Wt);
        wlagrange3(xp, mp, Wp);
        for (int m1 = 0; m1 < 3; m1++)
            for (int m2 = 0; m2 < 3; m2++) {
                iw[9 * i + 3 * m1 + m2] = Wt[m2] * Wp[m1];
                iidx[9 * i + 3 * m1 + m2] = V[3 * m1 + m2] - 1;
            }
    }
}

/* standalone interpolation table for two sample grids (for the known-answer test) */
void ora_interp_table(int Lcoarse, int Lfine, double* iw, int* iidx) {
    Level a = {0}, b = {0};
    a.L = a.nth = Lcoarse; a.nph = 2 * Lcoarse; a.K = a.nth * a.nph;
    b.L = b.nth = Lfine; b.nph = 2 * Lfine; b.K = b.nth * b.nph;
    fill_kappas(&a); fill_kappas(&b);
    build_interp(&a, &b, iw, iidx);
    free(a.kap); free(a.ath); free(a.aph); free(a.ang); free(a.wq);
    free(b.kap); free(b.ath); free(b.aph); free(b.ang); free(b.wq);
}

/* calcRad (maxPrecision = .false.), modMLFMA.f90:584-703 (used branch 661-697) */
static void calc_rad(Ctx* c) {
    Level* L = &c->lv[c->nlev];
    int K = L->K;
    c->frad = xcalloc((size_t)c->N * 2 * K, sizeof(cplx));
    double ka = (2. * PI) / c->ph.lambda;
#pragma omp parallel for schedule(dynamic, 4)
    for (int b = 0; b < L->nb; b++) {
        const double* C = L->centre + 3 * b;
        for (int t = c->box_ptr[b]; t < c->box_ptr[b + 1]; t++) {
            int n = c->box_bases[t];
            const double* bp = c->t_baric + 3 * c->e_t[2 * n + 0];
            const double* vp = c->p_coord + 3 * c->e_po[2 * n + 0];
            const double* bm = c->t_baric + 3 * c->e_t[2 * n + 1];
            const double* vm = c->p_coord + 3 * c->e_po[2 * n + 1];
            double lon = c->e_long[n];
            double rp[3], rm[3], dp[3], dm[3];
            for (int d = 0; d < 3; d++) { rp[d] = bp[d] - vp[d]; rm[d] = vm[d] - bm[d]; dp[d] = bp[d] - C[d]; dm[d] = bm[d] - C[d]; }
            cplx* out = c->frad + (size_t)n * 2 * K;
            for (int j = 0; j < K; j++) {
                const double* kk = L->kap + 3 * j;
                double ap = ka * (kk[0] * dp[0] + kk[1] * dp[1] + kk[2] * dp[2]);
                double am = ka * (kk[0] * dm[0] + kk[1] * dm[1] + kk[2] * dm[2]);
                cplx ep = cos(ap) + I * sin(ap), em = cos(am) + I * sin(am);
                cplx vt[3];
                for (int d = 0; d < 3; d++) vt[d] = ((ep * rp[d] + em * rm[d]) * lon) * 0.5;
                const double* at = L->ath + 3 * j;
                const double* af = L->aph + 3 * j;
                out[j] = vt[0] * at[0] + vt[1] * at[1] + vt[2] * at[2];
                out[K + j] = vt[0] * af[0] + vt[1] * af[1] + vt[2] * af[2];
            }
        }
    }
}

/* green, modGlobalMetod.f90:472-487 */
static inline cplx green(const Phys* ph, const double* a, const double* b) {
    double d0 = a[0] - b[0], d1 = a[1] - b[1], d2 = a[2] - b[2];
    double r = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
    double arg = ph->w * ph->smue * r;
    return (cos(arg) / r) + I * (-sin(arg) / r);
}

/* Zmn_MoM, modMoM.f90:85-128 */
static cplx zmn(const Ctx* c, int m, int n) {
    const Phys* ph = &c->ph;
    cplx AP[3] = {0, 0, 0}, AM[3] = {0, 0, 0}, PhiP = 0, PhiM = 0;
    const double* cpm = c->t_baric + 3 * c->e_t[2 * m + 0];
    const double* cmm = c->t_baric + 3 * c->e_t[2 * m + 1];
    int tpn = c->e_t[2 * n + 0], tmn = c->e_t[2 * n + 1];
    const double* vpn = c->p_coord + 3 * c->e_po[2 * n + 0];
    const double* vmn = c->p_coord + 3 * c->e_po[2 * n + 1];
    for (int i = 0; i < 9; i++) {
        const double* sp = c->t_baric_sub + 27 * tpn + 3 * i;
        const double* sm = c->t_baric_sub + 27 * tmn + 3 * i;
        cplx g11 = green(ph, cpm, sp), g12 = green(ph, cpm, sm);
        cplx g21 = green(ph, cmm, sp), g22 = green(ph, cmm, sm);
        for (int d = 0; d < 3; d++) {
            double r1 = sp[d] - vpn[d], r2 = vmn[d] - sm[d];
            AP[d] = AP[d] + ((g11 * r1) + (g12 * r2));
            AM[d] = AM[d] + ((g21 * r1) + (g22 * r2));
        }
        PhiP = PhiP + (g11 - g12);
        PhiM = PhiM + (g21 - g22);
    }
    double c72 = (double)(1.0f / 72.0f);
    double ln = c->e_long[n], lm = c->e_long[m];
    for (int d = 0; d < 3; d++) {
        AP[d] = ((AP[d] * (MU / PI)) * c72) * ln;
        AM[d] = ((AM[d] * (MU / PI)) * c72) * ln;
    }
    double den = ((36 * PI) * ph->w) * EPSI; /* jj*36*pi*w*epsi = (0, den) */
    cplx tP = ((-1.) * PhiP) * ln, tM = ((-1.) * PhiM) * ln;
    PhiP = (cimag(tP) / den) + I * (-creal(tP) / den);
    PhiM = (cimag(tM) / den) + I * (-creal(tM) / den);
    const double* vpm = c->p_coord + 3 * c->e_po[2 * m + 0];
    const double* vmm = c->p_coord + 3 * c->e_po[2 * m + 1];
    cplx s1 = 0, s2 = 0;
    for (int d = 0; d < 3; d++) s1 = s1 + AP[d] * (cpm[d] - vpm[d]);
    for (int d = 0; d < 3; d++) s2 = s2 + AM[d] * (-cmm[d] + vmm[d]);
    double fa = (0.5 * ph->w) * lm;     /* jj*0.5*w*e_long(m) = (0, fa) */
    cplx sum = s1 + s2;
    cplx PintA = (-fa * cimag(sum)) + I * (fa * creal(sum));
    cplx PintPhi = lm * (PhiM - PhiP);
    return PintPhi + PintA;
}

/* llenarZesparcida, modMLFMA.f90:1594-1634: CSR over rows 1..N, row m takes
 * the sorted near list of its leaf box; values rounded to complex(4). */
static void fill_near(Ctx* c) {
    int N = c->N;
    c->ia = xcalloc(N + 1, sizeof(int));
    for (int m = 0; m < N; m++) {
        int b = c->box_of[m];
        c->ia[m + 1] = c->ia[m] + (c->near_ptr[b + 1] - c->near_ptr[b]);
    }
    c->nnz = c->ia[N];
    c->ja = xcalloc(c->nnz, sizeof(int));
    c->zn = xcalloc(c->nnz, sizeof(cplxf));
#pragma omp parallel for schedule(dynamic, 16)
    for (int m = 0; m < N; m++) {
        int b = c->box_of[m];
        int64_t o = c->ia[m];
        for (int t = c->near_ptr[b]; t < c->near_ptr[b + 1]; t++, o++) {
            int n = c->near_bases[t];
            cplx z = zmn(c, m, n);
            c->ja[o] = n;
            c->zn[o] = (float)creal(z) + I * (float)cimag(z);
        }
    }
}

static void free_level(Level* L) {
    free(L->centre); free(L->parent); free(L->child_ptr);
    free(L->kap); free(L->ath); free(L->aph); free(L->ang); free(L->wq);
    free(L->far_ptr); free(L->far_src); free(L->far_tid); free(L->rab); free(L->T);
    free(L->iw); free(L->iidx); free(L->C); free(L->B); free(L->A);
}

void ora_free(Ctx* c) {
    if (!c) return;
    for (int n = 1; n <= c->nlev && n < 32; n++) free_level(&c->lv[n]);
    free(c->box_ptr); free(c->box_bases); free(c->box_of); free(c->near_ptr); free(c->near_bases);
    free(c->frad); free(c->ia); free(c->ja); free(c->zn); free(c->alu); free(c->jlu); free(c->ju);
    free(c->minv);
    free(c);
}

/* inicializar_MLFMA, modMLFMA.f90:113-275.  Geometry arrays are 0-based:
 * e_t[N][2], e_po[N][2] index triangles / nodes; coordinates row-major.
 * status: 0 ok, -1 body too small (nivel_max <= 3), -10 more than 316
 * unique displacements on a level. */
Ctx* ora_create(int N, int T, int P, const double* p_coord, const double* t_baric,
                const double* t_baric_sub, const double* e_long, const double* e_centro,
                const int* e_t, const int* e_po, double lambda, double ladomax,
                int legendre_mode, int* status) {
    Ctx* c = xcalloc(1, sizeof(Ctx));
    c->ph = phys_from_lambda(lambda);
    c->ladomax = ladomax;
    c->legendre_mode = legendre_mode;
    c->N = N; c->T = T; c->P = P;
    c->p_coord = p_coord; c->t_baric = t_baric; c->t_baric_sub = t_baric_sub;
    c->e_long = e_long; c->e_centro = e_centro; c->e_t = e_t; c->e_po = e_po;
    c->ilu_status = -1;
    int lim[6];
    limites(e_centro, N, lim);
    double maxX = e_centro[3 * lim[0]], minX = e_centro[3 * lim[1]];
    double maxY = e_centro[3 * lim[2] + 1], minY = e_centro[3 * lim[3] + 1];
    double maxZ = e_centro[3 * lim[4] + 2], minZ = e_centro[3 * lim[5] + 2];
    double dX = maxX - minX, dY = maxY - minY, dZ = maxZ - minZ;
    double roo[3] = {0.5 * (maxX + minX), 0.5 * (maxY + minY), 0.5 * (maxZ + minZ)};
    double lado;
    if (dX >= dY && dX >= dZ) lado = dX;
    else if (dY >= dX && dY >= dZ) lado = dY;
    else lado = dZ;
    double tol = lambda / 10000.;
    lado = lado + tol;
    double log2f_ = (double)log10f(2.0f);
    int nl = (int)ceil(1. + (log10(lado / (ladomax * lambda)) / log2f_));
    c->nlev = nl;
    memcpy(c->root_centre, roo, sizeof(roo));
    c->root_side = lado;
    if (nl <= 3 || nl >= 31) { *status = -1; return c; }
    double s3 = (double)sqrtf(3.0f), third = (double)(1.0f / 3.0f);
    for (int i = 1; i <= nl; i++) {
        Level* L = &c->lv[i];
        L->side = lado / ldexp(1.0, i - 1);
        double d = s3 * L->side;
        double kd = (2. * PI / lambda) * d;
        L->L = (int)floor(kd + 6 * pow(kd, third));
        L->nth = L->L; L->nph = 2 * L->L; L->K = L->nth * L->nph;
        if (i >= 3) fill_kappas(L);
    }
    lv_append(&c->lv[1], roo, -1);
    int* all = malloc(sizeof(int) * N);
    for (int i = 0; i < N; i++) all[i] = i;
    IVec lb = {0}, lp = {0};
    iv_push(&lp, 0);
    geom(c, roo, lado, all, N, 1, &lb, &lp);
    free(all);
    c->box_bases = lb.b; c->box_ptr = lp.b;
    Level* leaf = &c->lv[nl];
    c->box_of = malloc(sizeof(int) * N);
    for (int b = 0; b < leaf->nb; b++)
        for (int t = c->box_ptr[b]; t < c->box_ptr[b + 1]; t++) c->box_of[c->box_bases[t]] = b;
    /* children ranges (boxes of a parent are consecutive in depth-first order) */
    for (int i = 1; i < nl; i++) {
        Level* L = &c->lv[i];
        Level* Lc = &c->lv[i + 1];
        L->child_ptr = xcalloc(L->nb + 1, sizeof(int));
        for (int b = 0; b < Lc->nb; b++) L->child_ptr[Lc->parent[b] + 1]++;
        for (int b = 0; b < L->nb; b++) L->child_ptr[b + 1] += L->child_ptr[b];
    }
    for (int i = 3; i <= nl; i++) {
        Level* L = &c->lv[i];
        size_t sz = (size_t)L->nb * 2 * L->K;
        L->C = xcalloc(sz, sizeof(cplx)); L->B = xcalloc(sz, sizeof(cplx)); L->A = xcalloc(sz, sizeof(cplx));
    }
    calc_rad(c);
    int st = build_lists(c);
    if (st) { *status = st; return c; }
    fill_trans(c);
    fill_near(c);
    for (int n = 3; n < nl; n++) {
        Level* L = &c->lv[n];
        L->iw = malloc(sizeof(double) * 9 * L->K);
        L->iidx = malloc(sizeof(int) * 9 * L->K);
        build_interp(L, &c->lv[n + 1], L->iw, L->iidx);
    }
    *status = 0;
    return c;
}

/* inicializar_FMM, geomFMM, buscarFuncBases, hallar_n_multipolos_muestras,
 * llenar_functransf (modFMM.f90:170-268, 278-469, 479-490, 650-778): the
 * single-level FMM as a one-level tree (level 3 of this context, nlev = 3),
 * so calc_rad, fill_trans, fill_near and ora_matvec (which receives from B
 * when nlev = 3) apply unchanged.  Box side: ladomayor / ceiling(ladomayor /
 * (side_lambda * lambda)); the reference uses side_lambda = 1/2
 * (criterio_ladoW = lambda/2).  Boxes are visited z-major, then y, then x,
 * from the corner (max + tol/2) downwards with offsets accumulated by
 * repeated addition, and a basis belongs to the first box whose closed
 * bounds contain its edge centre.  Far: |c_i - c_j| >= 2 side - lambda/100;
 * displacements are deduplicated in order of first appearance (keyed here by
 * their integer grid offsets, which the reference's lambda/100 tolerance
 * identifies the same way).  Near rows: union of the near boxes' bases,
 * sorted ascending as the MLFMA rows are (the reference keeps box order,
 * which changes only the near sum's rounding). */
Ctx* ora_create_fmm(int N, int T, int P, const double* p_coord, const double* t_baric,
                    const double* t_baric_sub, const double* e_long, const double* e_centro,
                    const int* e_t, const int* e_po, double lambda, double side_lambda,
                    int legendre_mode, int* status) {
    Ctx* c = xcalloc(1, sizeof(Ctx));
    c->ph = phys_from_lambda(lambda);
    c->ladomax = side_lambda;
    c->legendre_mode = legendre_mode;
    c->N = N; c->T = T; c->P = P;
    c->p_coord = p_coord; c->t_baric = t_baric; c->t_baric_sub = t_baric_sub;
    c->e_long = e_long; c->e_centro = e_centro; c->e_t = e_t; c->e_po = e_po;
    c->ilu_status = -1;
    int lim[6];
    limites(e_centro, N, lim);
    double maxX = e_centro[3 * lim[0]], minX = e_centro[3 * lim[1]];
    double maxY = e_centro[3 * lim[2] + 1], minY = e_centro[3 * lim[3] + 1];
    double maxZ = e_centro[3 * lim[4] + 2], minZ = e_centro[3 * lim[5] + 2];
    double dX = maxX - minX, dY = maxY - minY, dZ = maxZ - minZ;
    double mayor;
    if (dX >= dY && dX >= dZ) mayor = dX;
    else if (dY >= dX && dY >= dZ) mayor = dY;
    else mayor = dZ;
    double tol = lambda / 10000.;
    mayor = mayor + tol;
    tol = tol / 2.;
    double corner[3] = {maxX + tol, maxY + tol, maxZ + tol};
    int ne = (int)ceil(mayor / (side_lambda * lambda));
    double lado = mayor / ne;
    c->nlev = 3;
    c->root_side = mayor;
    Level* L = &c->lv[3];
    L->side = lado;
    double s3 = (double)sqrtf(3.0f), third = (double)(1.0f / 3.0f);
    double kd = (2. * PI / lambda) * (s3 * lado);
    L->L = (int)floor(kd + 6 * pow(kd, third));
    L->nth = L->L; L->nph = 2 * L->L; L->K = L->nth * L->nph;
    fill_kappas(L);
    /* geomFMM: boxes in loop order, each takes the remaining bases inside it */
    int* rem = malloc(sizeof(int) * N);
    int* rest = malloc(sizeof(int) * N);
    for (int i = 0; i < N; i++) rem[i] = i;
    int nrem = N;
    IVec lb = {0}, lp = {0};
    iv_push(&lp, 0);
    double dz = 0.;
    for (int i = 0; i < ne; i++) {
        double dy = 0.;
        for (int j = 0; j < ne; j++) {
            double dx = 0.;
            for (int k = 0; k < ne; k++) {
                double esq[3] = {corner[0] - dx, corner[1] - dy, corner[2] - dz};
                double cen[3] = {esq[0] - lado / 2., esq[1] - lado / 2., esq[2] - lado / 2.};
                double lq = lado / 2.;
                double xmax = cen[0] + lq, xmin = cen[0] - lq, ymax = cen[1] + lq, ymin = cen[1] - lq;
                double zmax = cen[2] + lq, zmin = cen[2] - lq;
                int nf = 0, nr = 0;
                for (int t = 0; t < nrem; t++) {
                    const double* e = e_centro + 3 * rem[t];
                    if (e[0] <= xmax && e[0] >= xmin && e[1] <= ymax && e[1] >= ymin && e[2] <= zmax && e[2] >= zmin) {
                        iv_push(&lb, rem[t]);
                        nf++;
                    } else {
                        rest[nr++] = rem[t];
                    }
                }
                if (nf > 0) {
                    lv_append(L, cen, -1);
                    iv_push(&lp, lb.n);
                    memcpy(rem, rest, sizeof(int) * nr);
                    nrem = nr;
                }
                dx = dx + lado;
            }
            dy = dy + lado;
        }
        dz = dz + lado;
    }
    free(rem); free(rest);
    c->box_bases = lb.b; c->box_ptr = lp.b;
    c->box_of = malloc(sizeof(int) * N);
    for (int b = 0; b < L->nb; b++)
        for (int t = c->box_ptr[b]; t < c->box_ptr[b + 1]; t++) c->box_of[c->box_bases[t]] = b;
    size_t sz = (size_t)L->nb * 2 * L->K;
    L->C = xcalloc(sz, sizeof(cplx)); L->B = xcalloc(sz, sizeof(cplx)); L->A = xcalloc(sz, sizeof(cplx));
    calc_rad(c);
    /* llenar_functransf */
    double ftol = lambda / 100.;
    int span = 2 * ne - 1;
    int* tid_of = malloc(sizeof(int) * (size_t)span * span * span);
    for (size_t q = 0; q < (size_t)span * span * span; q++) tid_of[q] = -1;
    L->far_ptr = xcalloc(L->nb + 1, sizeof(int));
    IVec fs = {0}, ft = {0}, nearb = {0}, nearp = {0};
    iv_push(&nearp, 0);
    double* rab = NULL;
    int cont = 0;
    for (int i = 0; i < L->nb; i++) {
        int nstart = nearb.n;
        for (int j = 0; j < L->nb; j++) {
            double rh[3];
            for (int d = 0; d < 3; d++) rh[d] = L->centre[3 * i + d] - L->centre[3 * j + d];
            double nh = sqrt(rh[0] * rh[0] + rh[1] * rh[1] + rh[2] * rh[2]);
            if (nh >= 2 * lado - ftol) {
                int o[3];
                for (int d = 0; d < 3; d++) o[d] = (int)lround(rh[d] / lado) + ne - 1;
                size_t key = ((size_t)o[0] * span + o[1]) * span + o[2];
                int k = tid_of[key];
                if (k < 0) {
                    k = cont++;
                    tid_of[key] = k;
                    rab = realloc(rab, sizeof(double) * 3 * cont);
                    memcpy(rab + 3 * k, rh, sizeof(rh));
                }
                iv_push(&fs, j);
                iv_push(&ft, k);
            } else {
                for (int t = c->box_ptr[j]; t < c->box_ptr[j + 1]; t++) iv_push(&nearb, c->box_bases[t]);
            }
        }
        L->far_ptr[i + 1] = fs.n;
        int cnt = nearb.n - nstart;
        int* a = nearb.b + nstart;
        for (int t = 1; t < cnt; t++) {
            int v = a[t], q = t - 1;
            while (q >= 0 && a[q] > v) { a[q + 1] = a[q]; q--; }
            a[q + 1] = v;
        }
        iv_push(&nearp, nearb.n);
    }
    free(tid_of);
    L->far_src = fs.b ? fs.b : xcalloc(1, sizeof(int));
    L->far_tid = ft.b ? ft.b : xcalloc(1, sizeof(int));
    L->ntrans = cont;
    L->rab = rab ? rab : xcalloc(3, sizeof(double));
    c->near_ptr = nearp.b;
    c->near_bases = nearb.b;
    fill_trans(c);
    fill_near(c);
    *status = 0;
    return c;
}

/* ------------------------------------------------------------------ */
/* matvec                                                               */
/* ------------------------------------------------------------------ */

/* llenar_campoCyB, modMLFMA.f90:1783-1855 */
static void campo_cyb(Ctx* c, const cplx* x) {
    int nl = c->nlev;
    double k0 = (2. * PI) / c->ph.lambda;
    for (int n = 3; n <= nl; n++) {
        Level* L = &c->lv[n];
        memset(L->C, 0, sizeof(cplx) * (size_t)L->nb * 2 * L->K);
        memset(L->B, 0, sizeof(cplx) * (size_t)L->nb * 2 * L->K);
    }
    Level* leaf = &c->lv[nl];
    int K = leaf->K;
#pragma omp parallel for schedule(dynamic, 8)
    for (int b = 0; b < leaf->nb; b++) {
        cplx* Cb = leaf->C + (size_t)b * 2 * K;
        for (int t = c->box_ptr[b]; t < c->box_ptr[b + 1]; t++) {
            int n = c->box_bases[t];
            const cplx* R = c->frad + (size_t)n * 2 * K;
            for (int q = 0; q < 2 * K; q++) Cb[q] = Cb[q] + R[q] * x[n];
        }
    }
    for (int n = nl; n >= 4; n--) {
        Level* L = &c->lv[n];
        Level* Lp = &c->lv[n - 1];
        int Kp = Lp->K, Kc = L->K;
#pragma omp parallel for schedule(dynamic, 2)
        for (int p = 0; p < Lp->nb; p++) {
            cplx* Cp = Lp->C + (size_t)p * 2 * Kp;
            for (int cub = Lp->child_ptr[p]; cub < Lp->child_ptr[p + 1]; cub++) {
                double r[3];
                for (int d = 0; d < 3; d++) r[d] = L->centre[3 * cub + d] - Lp->centre[3 * p + d];
                const cplx* Cc = L->C + (size_t)cub * 2 * Kc;
                for (int m = 0; m < Kp; m++) {
                    const double* kk = Lp->kap + 3 * m;
                    double kr = kk[0] * r[0] + kk[1] * r[1] + kk[2] * r[2];
                    double a = k0 * kr;
                    cplx e = cos(a) + I * sin(a);
                    cplx v0 = 0, v1 = 0;
                    for (int t = 0; t < 9; t++) {
                        double w = Lp->iw[9 * m + t];
                        int ix = Lp->iidx[9 * m + t];
                        v0 = v0 + w * Cc[ix];
                        v1 = v1 + w * Cc[Kc + ix];
                    }
                    Cp[m] = Cp[m] + v0 * e;
                    Cp[Kp + m] = Cp[Kp + m] + v1 * e;
                }
            }
        }
    }
    for (int n = 3; n <= nl; n++) {
        Level* L = &c->lv[n];
        int Kn = L->K;
#pragma omp parallel for schedule(dynamic, 4)
        for (int b = 0; b < L->nb; b++) {
            cplx* Bb = L->B + (size_t)b * 2 * Kn;
            for (int f = L->far_ptr[b]; f < L->far_ptr[b + 1]; f++) {
                const cplx* Cs = L->C + (size_t)L->far_src[f] * 2 * Kn;
                const cplx* Tt = L->T + (size_t)L->far_tid[f] * Kn;
                for (int k = 0; k < Kn; k++) {
                    Bb[k] = Bb[k] + Cs[k] * Tt[k];
                    Bb[Kn + k] = Bb[Kn + k] + Cs[Kn + k] * Tt[k];
                }
            }
            for (int k = 0; k < Kn; k++) { Bb[k] = Bb[k] * L->wq[k]; Bb[Kn + k] = Bb[Kn + k] * L->wq[k]; }
        }
    }
}

/* llenar_campoA, modMLFMA.f90:1857-1897 */
static void campo_a(Ctx* c) {
    int nl = c->nlev;
    double k0 = (2. * PI) / c->ph.lambda;
    for (int n = 4; n <= nl; n++) {
        Level* L = &c->lv[n];
        Level* Lp = &c->lv[n - 1];
        int Kp = Lp->K, Kc = L->K;
        const cplx* Psrc = (n == 4) ? Lp->B : Lp->A;
#pragma omp parallel for schedule(dynamic, 4)
        for (int cub = 0; cub < L->nb; cub++) {
            int p = L->parent[cub];
            double r[3];
            for (int d = 0; d < 3; d++) r[d] = L->centre[3 * cub + d] - Lp->centre[3 * p + d];
            cplx* Ac = L->A + (size_t)cub * 2 * Kc;
            const cplx* Bc = L->B + (size_t)cub * 2 * Kc;
            cplx* ant = xcalloc(2 * (size_t)Kc, sizeof(cplx));
            const cplx* Pp = Psrc + (size_t)p * 2 * Kp;
            for (int m = 0; m < Kp; m++) {
                const double* kk = Lp->kap + 3 * m;
                double kr = kk[0] * r[0] + kk[1] * r[1] + kk[2] * r[2];
                double a = k0 * kr;
                cplx e = cos(a) - I * sin(a);
                cplx d0 = Pp[m] * e, d1 = Pp[Kp + m] * e;
                for (int t = 0; t < 9; t++) {
                    double w = Lp->iw[9 * m + t];
                    int ix = Lp->iidx[9 * m + t];
                    ant[ix] = ant[ix] + w * d0;
                    ant[Kc + ix] = ant[Kc + ix] + w * d1;
                }
            }
            for (int q = 0; q < 2 * Kc; q++) Ac[q] = Bc[q] + ant[q];
            free(ant);
        }
    }
}

/* MatxVec_MLFMA, modMLFMA.f90:1901-1946 */
void ora_matvec(Ctx* c, const cplx* x, cplx* y) {
    int nl = c->nlev;
    campo_cyb(c, x);
    campo_a(c);
    Level* leaf = &c->lv[nl];
    int K = leaf->K;
    const cplx* Aleaf = (nl == 3) ? leaf->B : leaf->A;
    cplx fac = I * c->ph.w * MU / (4. * PI);
#pragma omp parallel for schedule(dynamic, 8)
    for (int b = 0; b < leaf->nb; b++) {
        const cplx* Ab = Aleaf + (size_t)b * 2 * K;
        for (int t = c->box_ptr[b]; t < c->box_ptr[b + 1]; t++) {
            int n = c->box_bases[t];
            const cplx* R = c->frad + (size_t)n * 2 * K;
            cplx s = 0;
            /* sum(sum(funcREC*A, DIM=2), DIM=1) with funcREC = conjg(funcRAD) */
            for (int k = 0; k < K; k++) s = s + (conj(R[k]) * Ab[k] + conj(R[K + k]) * Ab[K + k]);
            y[n] = s * fac;
        }
    }
#pragma omp parallel for schedule(static)
    for (int m = 0; m < c->N; m++) {
        cplx s = y[m];
        for (int q = c->ia[m]; q < c->ia[m + 1]; q++) s = s + x[c->ja[q]] * (cplx)c->zn[q];
        y[m] = s;
    }
}

/* ------------------------------------------------------------------ */
/* ILU0 and its triangular solves                                       */
/* ------------------------------------------------------------------ */

/* complex(4) * complex(4) in single precision */
static inline cplxf cmulf(cplxf a, cplxf b) {
    float ar = crealf(a), ai = cimagf(a), br = crealf(b), bi = cimagf(b);
    float p1 = ar * br, p2 = ai * bi, p3 = ar * bi, p4 = ai * br;
    return (p1 - p2) + I * (p3 + p4);
}

/* ilu0C, modIterativo.f90:1805-1976 on a 1-based CSR (a, ja, ia), n rows.
 * Output MSR: alu(1:n) inverted diagonal, jlu(1)=n+2, ju(i) start of U.
 * Arrays are indexed 1-based (element 0 unused).  Returns ierr. */
int ora_ilu0_raw(int n, const cplxf* a, const int* ja, const int* ia, cplxf* alu, int* jlu, int* ju) {
    int* iw = xcalloc(n + 1, sizeof(int));
    int ju0 = n + 2;
    jlu[1] = ju0;
    for (int ii = 1; ii <= n; ii++) {
        int js = ju0;
        for (int j = ia[ii]; j <= ia[ii + 1] - 1; j++) {
            int jcol = ja[j];
            if (jcol == ii) {
                alu[ii] = a[j];
                iw[jcol] = ii;
                ju[ii] = ju0;
            } else {
                alu[ju0] = a[j];
                jlu[ju0] = ja[j];
                iw[jcol] = ju0;
                ju0 = ju0 + 1;
            }
        }
        jlu[ii + 1] = ju0;
        int jf = ju0 - 1;
        int jm = ju[ii] - 1;
        for (int j = js; j <= jm; j++) {
            int jrow = jlu[j];
            cplxf tlf = cmulf(alu[j], alu[jrow]);
            cplx tl = (double)crealf(tlf) + I * (double)cimagf(tlf);
            alu[j] = tlf;
            for (int jj = ju[jrow]; jj <= jlu[jrow + 1] - 1; jj++) {
                int jw = iw[jlu[jj]];
                if (jw != 0) {
                    cplx ajj = (double)crealf(alu[jj]) + I * (double)cimagf(alu[jj]);
                    cplx aw = (double)crealf(alu[jw]) + I * (double)cimagf(alu[jw]);
                    cplx r = aw - tl * ajj;
                    alu[jw] = (float)creal(r) + I * (float)cimag(r);
                }
            }
        }
        if (crealf(alu[ii]) == 0.0f && cimagf(alu[ii]) == 0.0f) { free(iw); return ii; }
        {
            double dr = crealf(alu[ii]), di = cimagf(alu[ii]);
            double den = dr * dr + di * di;
            double qr = dr / den, qi = -di / den;
            alu[ii] = (float)qr + I * (float)qi;
        }
        iw[ii] = 0;
        for (int i = js; i <= jf; i++) iw[jlu[i]] = 0;
    }
    free(iw);
    return 0;
}

/* lusol0C, modIterativo.f90:504-560 (1-based factor arrays, 0-based vectors) */
static void lusol0(int n, const cplx* y, cplx* x, const cplxf* alu, const int* jlu, const int* ju) {
    for (int i = 1; i <= n; i++) {
        cplx s = y[i - 1];
        for (int k = jlu[i]; k <= ju[i] - 1; k++)
            s = s - ((double)crealf(alu[k]) + I * (double)cimagf(alu[k])) * x[jlu[k] - 1];
        x[i - 1] = s;
    }
    for (int i = n; i >= 1; i--) {
        cplx s = x[i - 1];
        for (int k = ju[i]; k <= jlu[i + 1] - 1; k++)
            s = s - ((double)crealf(alu[k]) + I * (double)cimagf(alu[k])) * x[jlu[k] - 1];
        x[i - 1] = ((double)crealf(alu[i]) + I * (double)cimagf(alu[i])) * s;
    }
}

void ora_lusol0_raw(int n, const cplx* y, cplx* x, const cplxf* alu, const int* jlu, const int* ju) {
    lusol0(n, y, x, alu, jlu, ju);
}

/* bsort2C, modIterativo.f90:1673-1748: bubble passes moving the largest
 * moduli to the front until ncut positions are settled */
static void bsort2(cplx* w, int* ind, int n, int ncut) {
    int i = 1;
    for (;;) {
        int test = 0;
        for (int j = n - 1; j >= i; j--) {
            if (cabs(w[j - 1]) < cabs(w[j])) {
                cplx t = w[j - 1]; w[j - 1] = w[j]; w[j] = t;
                int q = ind[j - 1]; ind[j - 1] = ind[j]; ind[j] = q;
                test = 1;
            }
        }
        i++;
        if (!test || ncut < i) break;
    }
}

/* ilutC, modIterativo.f90:2432-2883 (dual threshold ILU as adapted to
 * complex by the reference; factors complex(4), work rows complex(8)).  The
 * reference's diagonal swap writes through a stale index (wu(j)); here the
 * diagonal is swapped into position 1.  Arrays 1-based like ora_ilu0_raw;
 * alu/jlu are grown as needed (returned through pointers). */
int ora_ilut_raw(int n, const cplxf* a, const int* ja, const int* ia, int lfil, double tol,
                 cplxf** alu_out, int** jlu_out, int* ju) {
    if (lfil < 0) return -4;
    size_t cap = (size_t)n + 2 + (size_t)ia[n + 1] * 2 + 16;
    cplxf* alu = xcalloc(cap, sizeof(cplxf));
    int* jlu = xcalloc(cap, sizeof(int));
    int* jr = xcalloc(n + 2, sizeof(int));
    int* jwl = xcalloc(n + 2, sizeof(int));
    int* jwu = xcalloc(n + 2, sizeof(int));
    cplx* wl = xcalloc(n + 2, sizeof(cplx));
    cplx* wu = xcalloc(n + 2, sizeof(cplx));
    double* unorm = xcalloc(n + 2, sizeof(double));
    long ju0 = n + 2;
    jlu[1] = (int)ju0;
    int ierr = 0;
    for (int ii = 1; ii <= n && !ierr; ii++) {
        int j1 = ia[ii], j2 = ia[ii + 1] - 1;
        int lenu = 0, lenl = 0;
        double tnorm = 0.0;
        for (int k = j1; k <= j2; k++) tnorm = tnorm + cabs((cplx)a[k]);
        tnorm = tnorm / (double)(j2 - j1 + 1);
        for (int j = j1; j <= j2; j++) {
            int k = ja[j];
            cplx t = (double)crealf(a[j]) + I * (double)cimagf(a[j]);
            if (tol * tnorm <= cabs(t)) {
                if (k < ii) { lenl++; jwl[lenl] = k; wl[lenl] = t; jr[k] = lenl; }
                else { lenu++; jwu[lenu] = k; wu[lenu] = t; jr[k] = lenu; }
            }
        }
        int lenl0 = lenl, lenu0 = lenu, jjj = 0, nl = 0;
        for (;;) {
            jjj++;
            if (lenl < jjj) break;
            int jrow = jwl[jjj], kk = jjj;
            for (int j = jjj + 1; j <= lenl; j++) if (jwl[j] < jrow) { jrow = jwl[j]; kk = j; }
            int jold = jwl[jjj];
            jwl[jjj] = jrow; jwl[kk] = jold;
            jr[jrow] = jjj; jr[jold] = kk;
            cplx sw = wl[kk]; wl[kk] = wl[jjj]; wl[jjj] = sw;
            if (ii <= jrow) break;
            cplx al = (double)crealf(alu[jrow]) + I * (double)cimagf(alu[jrow]);
            double fr = creal(wl[jjj]) * creal(al) - cimag(wl[jjj]) * cimag(al);
            double fi = creal(wl[jjj]) * cimag(al) + cimag(wl[jjj]) * creal(al);
            cplx fact = fr + I * fi;
            jr[jrow] = 0;
            if (cabs(fact) * unorm[jrow] <= tol * tnorm) continue;
            for (int k = ju[jrow]; k <= jlu[jrow + 1] - 1; k++) {
                double ar = crealf(alu[k]), ai = cimagf(alu[k]);
                cplx s = (fr * ar - fi * ai) + I * (fr * ai + fi * ar);
                int j = jlu[k];
                int jpos = jr[j];
                if (cabs(s) < tol * tnorm && jpos == 0) continue;
                if (ii <= j) {
                    if (jpos == 0) {
                        lenu++;
                        if (n < lenu) { ierr = -1; break; }
                        jwu[lenu] = j; jr[j] = lenu; wu[lenu] = -s;
                    } else wu[jpos] = wu[jpos] - s;
                } else {
                    if (jpos == 0) {
                        lenl++;
                        if (n < lenl) { ierr = -1; break; }
                        jwl[lenl] = j; jr[j] = lenl; wl[lenl] = -s;
                    } else wl[jpos] = wl[jpos] - s;
                }
            }
            if (ierr) break;
            nl++;
            wl[nl] = fact; jwl[nl] = jrow;
        }
        if (ierr) break;
        int len = nl < lenl0 + lfil ? nl : lenl0 + lfil;
        bsort2(wl + 1, jwl + 1, nl, len);
        if ((size_t)ju0 + len + lenu + 2 >= cap) {
            cap = 2 * cap + len + lenu + 16;
            alu = realloc(alu, cap * sizeof(cplxf));
            jlu = realloc(jlu, cap * sizeof(int));
        }
        for (int k = 1; k <= len; k++) {
            alu[ju0] = (float)creal(wl[k]) + I * (float)cimag(wl[k]);
            jlu[ju0] = jwl[k];
            ju0++;
        }
        ju[ii] = (int)ju0;
        for (int k = jjj; k <= lenl; k++) jr[jwl[k]] = 0;
        int idiag = jr[ii];
        if (idiag == 0) { ierr = ii; break; }
        if (idiag != 1) {
            cplx t = wu[1]; wu[1] = wu[idiag]; wu[idiag] = t;
            int q = jwu[1]; jwu[1] = jwu[idiag]; jwu[idiag] = q;
        }
        len = lenu < lenu0 + lfil ? lenu : lenu0 + lfil;
        bsort2(wu + 2, jwu + 2, lenu - 1, len);
        double t = 0.0;
        for (int k = 2; k <= len; k++) {
            jlu[ju0] = jwu[k];
            alu[ju0] = (float)creal(wu[k]) + I * (float)cimag(wu[k]);
            t = t + cabs(wu[k]);
            ju0++;
        }
        unorm[ii] = t / (double)(len + 1);
        if (cabs(wu[1]) == 0.0) { ierr = -5; break; }
        double dr = creal(wu[1]), di = cimag(wu[1]), den = dr * dr + di * di;
        alu[ii] = (float)(dr / den) + I * (float)(-di / den);
        jlu[ii + 1] = (int)ju0;
        for (int k = 1; k <= lenu; k++) jr[jwu[k]] = 0;
    }
    free(jr); free(jwl); free(jwu); free(wl); free(wu); free(unorm);
    *alu_out = alu;
    *jlu_out = jlu;
    return ierr;
}

int ora_ilut(Ctx* c, int lfil, double tol) {
    int n = c->N;
    int64_t nnz = c->nnz;
    cplxf* a1 = xcalloc(nnz + 1, sizeof(cplxf));
    int* ja1 = xcalloc(nnz + 1, sizeof(int));
    int* ia1 = xcalloc(n + 2, sizeof(int));
    for (int64_t q = 0; q < nnz; q++) { a1[q + 1] = c->zn[q]; ja1[q + 1] = c->ja[q] + 1; }
    for (int i = 0; i <= n; i++) ia1[i + 1] = c->ia[i] + 1;
    free(c->alu); free(c->jlu); free(c->ju);
    c->ju = xcalloc(n + 1, sizeof(int));
    c->ilu_status = ora_ilut_raw(n, a1, ja1, ia1, lfil, tol, &c->alu, &c->jlu, c->ju);
    free(a1); free(ja1); free(ia1);
    return c->ilu_status;
}

int64_t ora_ilu_len(Ctx* c) { return (int64_t)c->jlu[c->N + 1] - 1; }

/* crear_precond, ILU0 branch (main.f90:851-902) on the near CSR */
int ora_ilu0(Ctx* c) {
    int n = c->N;
    int64_t nnz = c->nnz;
    cplxf* a1 = xcalloc(nnz + 1, sizeof(cplxf));
    int* ja1 = xcalloc(nnz + 1, sizeof(int));
    int* ia1 = xcalloc(n + 2, sizeof(int));
    for (int64_t q = 0; q < nnz; q++) { a1[q + 1] = c->zn[q]; ja1[q + 1] = c->ja[q] + 1; }
    for (int i = 0; i <= n; i++) ia1[i + 1] = c->ia[i] + 1;
    free(c->alu); free(c->jlu); free(c->ju);
    c->alu = xcalloc(nnz + 2, sizeof(cplxf));
    c->jlu = xcalloc(nnz + 2, sizeof(int));
    c->ju = xcalloc(n + 1, sizeof(int));
    c->ilu_status = ora_ilu0_raw(n, a1, ja1, ia1, c->alu, c->jlu, c->ju);
    free(a1); free(ja1); free(ia1);
    return c->ilu_status;
}

void ora_lusol0(Ctx* c, const cplx* y, cplx* x) { lusol0(c->N, y, x, c->alu, c->jlu, c->ju); }

/* ------------------------------------------------------------------ */
/* neighbourhood-inverse preconditioner                                 */
/* ------------------------------------------------------------------ */

/* For every leaf box b with neighbourhood S (the sorted near list of b, the
 * column set of each of b's rows in the near CSR), A = Znear[S, S] (entries
 * absent from the CSR are zero).  The rows of A^-1 that belong to b's own
 * bases become the rows of M, so M has the near CSR's pattern and
 * M x = sum over boxes of (A^-1 x_S)[own].  Rows of A^-1 solve
 * A^T X = E_own (Gaussian elimination with partial pivoting, largest |a|^2,
 * first index on ties, in double).  This preconditioner is an addition of
 * this build (the reference offers ILU0/ILUT only); it is linear and fixed,
 * so right-preconditioned CGS stays valid.  Returns 0 or the first box whose
 * block is singular (+1). */
int ora_nearinv(Ctx* c) {
    Level* leaf = &c->lv[c->nlev];
    free(c->minv);
    c->minv = xcalloc(c->nnz, sizeof(cplx));
    int bad = 0;
#pragma omp parallel for schedule(dynamic, 4)
    for (int b = 0; b < leaf->nb; b++) {
        int m0 = c->box_bases[c->box_ptr[b]];
        int n = c->ia[m0 + 1] - c->ia[m0];
        const int* S = c->ja + c->ia[m0];
        int nown = c->box_ptr[b + 1] - c->box_ptr[b];
        cplx* At = xcalloc((size_t)n * n, sizeof(cplx));
        cplx* X = xcalloc((size_t)n * nown, sizeof(cplx));
        for (int r = 0; r < n; r++) {
            int m = S[r];
            for (int q = c->ia[m]; q < c->ia[m + 1]; q++) {
                int col = c->ja[q];
                int lo = 0, hi = n - 1, pos = -1;
                while (lo <= hi) {
                    int mid = (lo + hi) / 2;
                    if (S[mid] == col) { pos = mid; break; }
                    if (S[mid] < col) lo = mid + 1; else hi = mid - 1;
                }
                if (pos >= 0) At[(size_t)pos * n + r] = (double)crealf(c->zn[q]) + I * (double)cimagf(c->zn[q]);
            }
        }
        for (int i = 0; i < nown; i++) {
            int g = c->box_bases[c->box_ptr[b] + i];
            for (int j = 0; j < n; j++) if (S[j] == g) X[(size_t)j * nown + i] = 1.0;
        }
        int sing = 0;
        for (int k = 0; k < n && !sing; k++) {
            int piv = k;
            double best = -1.0;
            for (int i = k; i < n; i++) {
                cplx a = At[(size_t)i * n + k];
                double v = creal(a) * creal(a) + cimag(a) * cimag(a);
                if (v > best) { best = v; piv = i; }
            }
            if (best == 0.0) { sing = 1; break; }
            if (piv != k) {
                for (int j = 0; j < n; j++) { cplx t = At[(size_t)k * n + j]; At[(size_t)k * n + j] = At[(size_t)piv * n + j]; At[(size_t)piv * n + j] = t; }
                for (int j = 0; j < nown; j++) { cplx t = X[(size_t)k * nown + j]; X[(size_t)k * nown + j] = X[(size_t)piv * nown + j]; X[(size_t)piv * nown + j] = t; }
            }
            cplx d = At[(size_t)k * n + k];
            for (int i = k + 1; i < n; i++) {
                cplx f = At[(size_t)i * n + k] / d;
                if (f == 0) continue;
                for (int j = k + 1; j < n; j++) At[(size_t)i * n + j] -= f * At[(size_t)k * n + j];
                for (int j = 0; j < nown; j++) X[(size_t)i * nown + j] -= f * X[(size_t)k * nown + j];
            }
        }
        if (sing) {
#pragma omp critical
            { if (!bad || b + 1 < bad) bad = b + 1; }
        } else {
            for (int k = n - 1; k >= 0; k--) {
                cplx d = At[(size_t)k * n + k];
                for (int j = 0; j < nown; j++) X[(size_t)k * nown + j] /= d;
                for (int i = 0; i < k; i++) {
                    cplx f = At[(size_t)i * n + k];
                    for (int j = 0; j < nown; j++) X[(size_t)i * nown + j] -= f * X[(size_t)k * nown + j];
                }
            }
            for (int i = 0; i < nown; i++) {
                int g = c->box_bases[c->box_ptr[b] + i];
                for (int j = 0; j < n; j++) c->minv[c->ia[g] + j] = X[(size_t)j * nown + i];
            }
        }
        free(At); free(X);
    }
    return bad;
}

static void nearinv_apply(Ctx* c, const cplx* y, cplx* x) {
#pragma omp parallel for schedule(static)
    for (int m = 0; m < c->N; m++) {
        cplx s = 0;
        for (int q = c->ia[m]; q < c->ia[m + 1]; q++) s = s + c->minv[q] * y[c->ja[q]];
        x[m] = s;
    }
}

void ora_nearinv_apply(Ctx* c, const cplx* y, cplx* x) { nearinv_apply(c, y, x); }
void ora_nearinv_values(Ctx* c, cplx* out) { memcpy(out, c->minv, sizeof(cplx) * c->nnz); }

/* ------------------------------------------------------------------ */
/* CGS                                                                  */
/* ------------------------------------------------------------------ */

static double nrm2(const cplx* v, int n) {
    double s = 0;
    for (int i = 0; i < n; i++) s += creal(v[i]) * creal(v[i]) + cimag(v[i]) * cimag(v[i]);
    return sqrt(s);
}

/* CGSold, modIterativo.f90:331-493, with an iteration cap added.
 * matvec: this context's MLFMA matvec.  prec: 1 = ILU0 factors of the
 * context (ora_ilu0 must have succeeded), 2 = neighbourhood inverse
 * (ora_nearinv must have succeeded).  Returns 0 converged, 1 maxit,
 * 2 breakdown (rho == 0), 3 non-finite. */
int ora_cgs(Ctx* c, const cplx* b, const cplx* guess, double errmax, int maxit, int prec,
            cplx* x, int* iters, double* relres, double* hist) {
    int n = c->N;
    cplx *r = malloc(sizeof(cplx) * n), *R_ = malloc(sizeof(cplx) * n), *u = malloc(sizeof(cplx) * n);
    cplx *p = malloc(sizeof(cplx) * n), *P_ = malloc(sizeof(cplx) * n), *V_ = malloc(sizeof(cplx) * n);
    cplx *q = malloc(sizeof(cplx) * n), *U_ = malloc(sizeof(cplx) * n), *Q_ = malloc(sizeof(cplx) * n);
    cplx* tmp = malloc(sizeof(cplx) * n);
    ora_matvec(c, guess, tmp);
    for (int i = 0; i < n; i++) { r[i] = b[i] - tmp[i]; R_[i] = r[i]; x[i] = guess[i]; }
    double nb = nrm2(b, n);
    cplx rho1 = 0, rho2 = 0;
    int it = 0, status = 1;
    double rr = nrm2(r, n);
    while (it < maxit) {
        it++;
        cplx s = 0;
        for (int i = 0; i < n; i++) s = s + r[i] * R_[i];
        rho1 = s;
        if (rho1 == 0) { status = 2; it--; break; }
        if (!isfinite(creal(rho1)) || !isfinite(cimag(rho1))) { status = 3; break; }
        if (it == 1) {
            for (int i = 0; i < n; i++) { u[i] = r[i]; p[i] = u[i]; }
        } else {
            cplx beta = rho1 / rho2;
            for (int i = 0; i < n; i++) {
                u[i] = r[i] + (beta * q[i]);
                p[i] = u[i] + (beta * (q[i] + (beta * p[i])));
            }
        }
        if (prec == 1) lusol0(n, p, P_, c->alu, c->jlu, c->ju);
        else if (prec == 2) nearinv_apply(c, p, P_);
        else memcpy(P_, p, sizeof(cplx) * n);
        ora_matvec(c, P_, V_);
        cplx sv = 0;
        for (int i = 0; i < n; i++) sv = sv + R_[i] * V_[i];
        cplx alfa = rho1 / sv;
        for (int i = 0; i < n; i++) { q[i] = u[i] - (alfa * V_[i]); tmp[i] = u[i] + q[i]; }
        if (prec == 1) lusol0(n, tmp, U_, c->alu, c->jlu, c->ju);
        else if (prec == 2) nearinv_apply(c, tmp, U_);
        else memcpy(U_, tmp, sizeof(cplx) * n);
        for (int i = 0; i < n; i++) x[i] = x[i] + (alfa * U_[i]);
        ora_matvec(c, U_, Q_);
        for (int i = 0; i < n; i++) r[i] = r[i] - (alfa * Q_[i]);
        rr = nrm2(r, n);
        if (hist) hist[it - 1] = rr / nb;
        if (!isfinite(rr)) { status = 3; break; }
        if (rr < errmax * nb) { status = 0; break; }
        rho2 = rho1;
    }
    *iters = it;
    *relres = rr / nb;
    free(r); free(R_); free(u); free(p); free(P_); free(V_); free(q); free(U_); free(Q_); free(tmp);
    return status;
}

/* ------------------------------------------------------------------ */
/* excitation and RCS                                                   */
/* ------------------------------------------------------------------ */

/* generar_onda, main.f90:1488-1525 (alphaCFIE = 1 keeps only the E term).
 * pol[3] complex, ctte complex, dir[3] real. */
void ora_generar_onda(int N, const double* p_coord, const double* t_baric, const double* e_long,
                      const int* e_t, const int* e_po, double lambda, const double* dir,
                      const cplx* pol, double ctte_re, double ctte_im, cplx* res) {
    Phys ph = phys_from_lambda(lambda);
    cplx ctte = ctte_re + I * ctte_im;
    double nd = sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
    double u[3] = {dir[0] / nd, dir[1] / nd, dir[2] / nd};
    for (int i = 0; i < N; i++) {
        cplx acc = 0;
        for (int s = 0; s < 2; s++) {
            const double* bc = t_baric + 3 * e_t[2 * i + s];
            const double* vo = p_coord + 3 * e_po[2 * i + s];
            double a = (ph.w * ph.smue) * (u[0] * bc[0] + u[1] * bc[1] + u[2] * bc[2]);
            cplx e = cos(a) - I * sin(a);
            cplx sum = 0;
            for (int d = 0; d < 3; d++) {
                cplx oE = (pol[d] * ctte) * e;
                double arm = s == 0 ? bc[d] - vo[d] : vo[d] - bc[d];
                sum = sum + oE * arm;
            }
            acc = acc + sum;
        }
        res[i] = (acc * 0.5) * e_long[i];
    }
}

/* calc_RCS + calc_E + sigmaRCS, modRCS.f90:60-153.  Returns sigma (linear)
 * for each (theta, phi); pol and ctte as given to inicializar_RCS. */
void ora_rcs(int N, const double* t_baric, const double* e_long, const double* e_centro,
             const int* e_t, double lambda_in, const cplx* Icur, const cplx* pol, double ctte_re,
             double ctte_im, const double* theta, const double* phi, int nang, double* sigma) {
    Phys ph = phys_from_lambda(lambda_in);
    cplx ctte = ctte_re + I * ctte_im;
    int lim[6];
    limites(e_centro, N, lim);
    double maxX = e_centro[3 * lim[0]], minX = e_centro[3 * lim[1]];
    double maxY = e_centro[3 * lim[2] + 1], minY = e_centro[3 * lim[3] + 1];
    double maxZ = e_centro[3 * lim[4] + 2], minZ = e_centro[3 * lim[5] + 2];
    double lambda = 2 * PI / (ph.w * sqrt(MU * EPSI));
    double D = sqrt(((maxX - minX) * (maxX - minX)) + ((maxY - minY) * (maxY - minY)) + ((maxZ - minZ) * (maxZ - minZ)));
    double rzl = 2 * (D * D) / lambda;
    if (50 * D > rzl) rzl = 50 * D;
    if (20 * lambda > rzl) rzl = 20 * lambda;
    rzl = rzl * 10;
    double roo[3] = {0.5 * (maxX + minX), 0.5 * (maxY + minY), 0.5 * (maxZ + minZ)};
    double den = 0;
    for (int d = 0; d < 3; d++) { cplx v = pol[d] * ctte; den += creal(conj(v) * v); }
    cplx fac = I * ph.w * MU / (4 * PI);
#pragma omp parallel for schedule(dynamic)
    for (int a = 0; a < nang; a++) {
        double ro[3] = {roo[0] + (rzl * sin(theta[a]) * cos(phi[a])),
                        roo[1] + (rzl * sin(theta[a]) * sin(phi[a])),
                        roo[2] + (rzl * cos(theta[a]))};
        cplx E[3] = {0, 0, 0};
        for (int i = 0; i < N; i++) {
            const double* cp = t_baric + 3 * e_t[2 * i];
            const double* cm = t_baric + 3 * e_t[2 * i + 1];
            double rm[3], rrm[3];
            cplx m[3];
            for (int d = 0; d < 3; d++) {
                rm[d] = 0.5 * (cp[d] + cm[d]);
                m[d] = ((cm[d] - cp[d]) * Icur[i]) * e_long[i];
                rrm[d] = ro[d] - rm[d];
            }
            cplx mr = m[0] * rrm[0] + m[1] * rrm[1] + m[2] * rrm[2];
            double rr = rrm[0] * rrm[0] + rrm[1] * rrm[1] + rrm[2] * rrm[2];
            cplx g = green(&ph, ro, rm);
            for (int d = 0; d < 3; d++) E[d] = E[d] + (g * ((mr * rrm[d] / rr) - m[d]));
        }
        double s = 0;
        for (int d = 0; d < 3; d++) { cplx e = E[d] * fac; s += creal(conj(e) * e); }
        sigma[a] = s * 4 * PI * (rzl * rzl) / den;
    }
}

/* dense MoM matrix rows (llenarZ_MoM, modMoM.f90:61-82), for small cases */
void ora_zmn_block(Ctx* c, int m0, int m1, cplx* Z /* (m1-m0) x N row-major */) {
#pragma omp parallel for schedule(dynamic)
    for (int m = m0; m < m1; m++)
        for (int n = 0; n < c->N; n++) Z[(size_t)(m - m0) * c->N + n] = zmn(c, m, n);
}

/* ------------------------------------------------------------------ */
/* accessors                                                            */
/* ------------------------------------------------------------------ */

int ora_nlev(Ctx* c) { return c->nlev; }
int64_t ora_nnz(Ctx* c) { return c->nnz; }
void ora_level_info(Ctx* c, int n, int* out /* nb, L, K, ntrans, nfar */, double* side) {
    Level* L = &c->lv[n];
    out[0] = L->nb; out[1] = L->L; out[2] = L->K; out[3] = L->ntrans;
    out[4] = (n >= 3 && L->far_ptr) ? L->far_ptr[L->nb] : 0;
    *side = L->side;
}
void ora_level_centres(Ctx* c, int n, double* out) { memcpy(out, c->lv[n].centre, sizeof(double) * 3 * c->lv[n].nb); }
void ora_level_parents(Ctx* c, int n, int* out) { memcpy(out, c->lv[n].parent, sizeof(int) * c->lv[n].nb); }
void ora_level_far(Ctx* c, int n, int* ptr, int* src, int* tid) {
    Level* L = &c->lv[n];
    memcpy(ptr, L->far_ptr, sizeof(int) * (L->nb + 1));
    memcpy(src, L->far_src, sizeof(int) * L->far_ptr[L->nb]);
    memcpy(tid, L->far_tid, sizeof(int) * L->far_ptr[L->nb]);
}
void ora_level_trans(Ctx* c, int n, double* rab, cplx* T) {
    Level* L = &c->lv[n];
    memcpy(rab, L->rab, sizeof(double) * 3 * L->ntrans);
    memcpy(T, L->T, sizeof(cplx) * (size_t)L->ntrans * L->K);
}
void ora_level_interp(Ctx* c, int n, double* iw, int* iidx) {
    Level* L = &c->lv[n];
    memcpy(iw, L->iw, sizeof(double) * 9 * L->K);
    memcpy(iidx, L->iidx, sizeof(int) * 9 * L->K);
}
void ora_level_fields(Ctx* c, int n, cplx* C, cplx* B, cplx* A) {
    Level* L = &c->lv[n];
    size_t sz = sizeof(cplx) * (size_t)L->nb * 2 * L->K;
    if (C) memcpy(C, L->C, sz);
    if (B) memcpy(B, L->B, sz);
    if (A) memcpy(A, L->A, sz);
}
void ora_leaf_boxes(Ctx* c, int* box_ptr, int* box_bases) {
    Level* L = &c->lv[c->nlev];
    memcpy(box_ptr, c->box_ptr, sizeof(int) * (L->nb + 1));
    memcpy(box_bases, c->box_bases, sizeof(int) * c->N);
}
void ora_patterns(Ctx* c, cplx* out) { memcpy(out, c->frad, sizeof(cplx) * (size_t)c->N * 2 * c->lv[c->nlev].K); }
void ora_near(Ctx* c, int* ia, int* ja, cplxf* z) {
    memcpy(ia, c->ia, sizeof(int) * (c->N + 1));
    memcpy(ja, c->ja, sizeof(int) * c->nnz);
    memcpy(z, c->zn, sizeof(cplxf) * c->nnz);
}
void ora_ilu_factors(Ctx* c, cplxf* alu, int* jlu, int* ju) {
    int64_t len = (int64_t)c->jlu[c->N + 1] + 1;
    memcpy(alu, c->alu, sizeof(cplxf) * len);
    memcpy(jlu, c->jlu, sizeof(int) * len);
    memcpy(ju, c->ju, sizeof(int) * (c->N + 1));
}
/* replace the near-field values (same CSR pattern), e.g. with values computed
 * elsewhere, so that later stages can be compared in isolation */
void ora_set_near(Ctx* c, const cplxf* z) { memcpy(c->zn, z, sizeof(cplxf) * c->nnz); }
double ora_root(Ctx* c, double* centre) { memcpy(centre, c->root_centre, sizeof(double) * 3); return c->root_side; }
void ora_set_threads(int n) {
#ifdef _OPENMP
    omp_set_num_threads(n);
#else
    (void)n;
#endif
}
int ora_get_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
