/* CPU oracle: precompute, trace loop, detector scoring (test infrastructure only).
 *
 * Plain-C restatement of the reference's hot path (file CLARITAS/CLARITAS.py):
 *   precompute  _prepare_gpu_particle_physics :6036-6965 and its kernels
 *               (PSD normalisation :3607-3635, Mie :3488-3592, rates :3845-3921,
 *               sediment :3925-4038, meridional field solver :4040-4220 driven as
               in :6451-6725, or the finalisation :4203-4220 of a supplied grid)
 *   transport   trace_kernel :4551-5104
 *   detectors   score_detectors_kernel :4378-4436 and helpers :4237-4376
 * The physics helpers live in oracle_transport_a.h / oracle_transport_b.h.
 * Of the observational outputs of the reference that never feed a transport decision, the per-ray
 * provenance (first/last bin, event type and deflection, acrylic returns; clo_trace_provenance) is
 * restated; the light-history grids, heatmaps, the particle_diag_* arrays and the remaining per-ray
 * histories are not. Built with -ffp-contract=off (oracle/Makefile).
 */
#define _GNU_SOURCE
#include "claritas_oracle.h"
#include "oracle_transport_b.h"
#include "tally_extras.h"

#include <stdio.h>
#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#endif

struct clo_state {
    clr_scene_params sp;
    int n, nt, n_radial, grid_nr, grid_nz;
    float grid_zmax;
    double *d, *wd, *nidx, *kidx;
    int* nstop;
    double *x, *qext, *qsca, *qabs, *qback, *g, *albedo;
    double *theta, *phase_cdf;
    double *radius, *nden, *mug, *mus, *mue, *muw, *muev, *gcdf, *wcdf, *pcdf, *muscal;
    double *moment_a, *moment_b;
    unsigned char* moment_mode;
    double *trace_geom, *trace_wave;
    double *sed_A, *sed_B, *sed_norm, *sed_max, *sed_radial_log, *sed_major, *sed_grid;
    double *sed_ws, *sed_wr;        /* settling velocity [n], radial slip table [n][n_radial] */
    int solver_iterations;          /* meridional solver: iterations done, largest residual at the last check */
    double solver_residual;
    char err[256];
};

static double* zalloc(size_t n) { return (double*)calloc(n ? n : 1, sizeof(double)); }

const char* clo_last_error(clo_state* s) { return s ? s->err : "null state"; }
double clo_erfinv(double y) { return oracle_erfinv(y); }

void clo_free(clo_state* s) {
    if (!s) return;
    double* arrs[] = {s->d, s->wd, s->nidx, s->kidx, s->x, s->qext, s->qsca, s->qabs, s->qback, s->g, s->albedo,
                      s->theta, s->phase_cdf, s->radius, s->nden, s->mug, s->mus, s->mue, s->muw, s->muev, s->gcdf,
                      s->wcdf, s->pcdf, s->muscal, s->moment_a, s->moment_b, s->trace_geom, s->trace_wave, s->sed_A,
                      s->sed_B, s->sed_norm, s->sed_max, s->sed_radial_log, s->sed_major, s->sed_grid,
                      s->sed_ws, s->sed_wr};
    for (size_t i = 0; i < sizeof arrs / sizeof arrs[0]; ++i) free(arrs[i]);
    free(s->nstop);
    free(s->moment_mode);
    free(s);
}

/* ---------------- FP64 complex helpers for the Mie series (:1138-1146) ---------------- */
typedef struct { double re, im; } cd_t;
static inline cd_t cd(double re, double im) { cd_t z; z.re = re; z.im = im; return z; }
static inline cd_t cd_add(cd_t a, cd_t b) { return cd(a.re + b.re, a.im + b.im); }
static inline cd_t cd_sub(cd_t a, cd_t b) { return cd(a.re - b.re, a.im - b.im); }
static inline cd_t cd_mul(cd_t a, cd_t b) { return cd(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
static inline cd_t cd_scale(cd_t a, double s) { return cd(a.re * s, a.im * s); }
static inline cd_t cd_div(cd_t a, cd_t b) {
    double d = b.re * b.re + b.im * b.im;
    if (d < 1e-300) d = 1e-300;
    return cd((a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d);
}
static inline double cd_abs2(cd_t a) { return a.re * a.re + a.im * a.im; }
static inline double cd_rmc(cd_t a, cd_t b) { return a.re * b.re + a.im * b.im; }

/* Mie coefficients and efficiencies for one bin (:3495-3559). a/b receive nstop terms. */
static int mie_bin(double diameter, double n_real, double k_imag, double n_medium, double wavelength, cd_t* D,
                   cd_t* a, cd_t* b, int* nstop_out, double* xo, double* qe_o, double* qs_o, double* qa_o,
                   double* qb_o, double* g_o, double* alb_o) {
    double x = O_PI_D * n_medium * diameter / wavelength;
    *xo = x;
    if (!(x > 0.0) || !(n_real > 0.0) || !(n_medium > 0.0) || !(wavelength > 0.0)) {
        *nstop_out = 0; *qe_o = *qs_o = *qa_o = *qb_o = *g_o = 0.0; *alb_o = 1.0;
        return 2;
    }
    double mr = n_real / n_medium, mi = k_imag / n_medium;
    int nstop = (int)(x + 4.0 * cbrt(x) + 2.0);
    if (nstop < 1) nstop = 1;
    double mz = hypot(mr * x, mi * x);
    int nmx = (int)fmax((double)nstop, mz) + 128;
    if (nmx < nstop + 1) nmx = nstop + 1;
    if (nmx >= CLR_MIE_MAX_ORDER || nstop >= CLR_MIE_MAX_ORDER) { *nstop_out = 0; return 1; }
    *nstop_out = nstop;
    D[nmx] = cd(0.0, 0.0);
    cd_t z = cd(mr * x, mi * x);
    for (int n = nmx; n >= 1; --n) {
        cd_t nz = cd_div(cd((double)n, 0.0), z);
        D[n - 1] = cd_sub(nz, cd_div(cd(1.0, 0.0), cd_add(D[n], nz)));
    }
    double psi_nm1 = sin(x), psi_n = sin(x) / x - cos(x);
    double chi_nm1 = cos(x), chi_n = cos(x) / x + sin(x);
    cd_t m = cd(mr, mi);
    for (int j = 0; j < nstop; ++j) {
        int n = j + 1;
        cd_t xi_nm1 = cd(psi_nm1, -chi_nm1), xi_n = cd(psi_n, -chi_n);
        cd_t dn = D[n];
        cd_t ca = cd_add(cd_div(dn, m), cd((double)n / x, 0.0));
        cd_t cb = cd_add(cd_mul(m, dn), cd((double)n / x, 0.0));
        a[j] = cd_div(cd_sub(cd_scale(ca, psi_n), cd(psi_nm1, 0.0)), cd_sub(cd_mul(ca, xi_n), xi_nm1));
        b[j] = cd_div(cd_sub(cd_scale(cb, psi_n), cd(psi_nm1, 0.0)), cd_sub(cd_mul(cb, xi_n), xi_nm1));
        double psi_np1 = ((2.0 * n + 1.0) / x) * psi_n - psi_nm1;
        double chi_np1 = ((2.0 * n + 1.0) / x) * chi_n - chi_nm1;
        psi_nm1 = psi_n; psi_n = psi_np1; chi_nm1 = chi_n; chi_n = chi_np1;
    }
    double se = 0.0, ss = 0.0, sbr = 0.0, sbi = 0.0, t1 = 0.0, t2 = 0.0;
    for (int j = 0; j < nstop; ++j) {
        int n = j + 1;
        double cn = 2.0 * n + 1.0;
        cd_t aa = a[j], bb = b[j];
        se += cn * (aa.re + bb.re);
        ss += cn * (cd_abs2(aa) + cd_abs2(bb));
        double sign = (n & 1) ? -1.0 : 1.0;
        sbr += cn * sign * (aa.re - bb.re);
        sbi += cn * sign * (aa.im - bb.im);
        t2 += (cn / ((double)n * (n + 1.0))) * cd_rmc(aa, bb);
        if (j + 1 < nstop) t1 += ((double)n * (n + 2.0) / (n + 1.0)) * (cd_rmc(aa, a[j + 1]) + cd_rmc(bb, b[j + 1]));
    }
    double x2 = x * x;
    double qe = 2.0 * se / x2, qs = 2.0 * ss / x2, qb = (sbr * sbr + sbi * sbi) / x2;
    if (qe < 0.0 && qe > -1e-12) qe = 0.0;
    if (qs < 0.0 && qs > -1e-12) qs = 0.0;
    double qa = qe - qs;
    if (qa < 0.0 && qa > -1e-10) qa = 0.0;
    double gg = qs > 0.0 ? 4.0 * (t1 + t2) / (x2 * qs) : 0.0;
    if (gg > 1.0) gg = 1.0;
    if (gg < -1.0) gg = -1.0;
    *qe_o = qe; *qs_o = qs; *qa_o = qa; *qb_o = qb; *g_o = gg; *alb_o = qe > 0.0 ? qs / qe : 1.0;
    return 0;
}

/* S1/S2 phase pdf * sin(theta) for one (bin, angle) (:3561-3581) */
static double mie_pdf(double th, int nstop, const cd_t* a, const cd_t* b) {
    double mu = cos(th), s1r = 0.0, s1i = 0.0, s2r = 0.0, s2i = 0.0, pi_nm1 = 0.0, pi_n = 1.0;
    for (int k = 0; k < nstop; ++k) {
        int n = k + 1;
        double nf = (double)n;
        double tau = nf * mu * pi_n - (nf + 1.0) * pi_nm1;
        double c = (2.0 * nf + 1.0) / (nf * (nf + 1.0));
        double ar = a[k].re, ai = a[k].im, br = b[k].re, bi = b[k].im;
        s1r += c * (ar * pi_n + br * tau);
        s1i += c * (ai * pi_n + bi * tau);
        s2r += c * (ar * tau + br * pi_n);
        s2i += c * (ai * tau + bi * pi_n);
        double pi_np1 = ((2.0 * nf + 1.0) / nf) * mu * pi_n - ((nf + 1.0) / nf) * pi_nm1;
        pi_nm1 = pi_n; pi_n = pi_np1;
    }
    double intensity = 0.5 * (s1r * s1r + s1i * s1i + s2r * s2r + s2i * s2i);
    return intensity * sin(th);
}

/* Schiller-Naumann settling velocity by damped Newton (:3925-3937) */
static double schiller_naumann(double v0, double d, double rho_w, double mu, double* out_Re, double* out_drag) {
    if (!(v0 > 0.0)) { *out_Re = 0.0; *out_drag = 1.0; return 0.0; }
    double v = v0, K = rho_w * d / mu;
    for (int it = 0; it < 24; ++it) {
        double Re = fmax(K * v, 0.0);
        double corr = 0.15 * pow(Re, 0.687);
        double f = v * (1.0 + corr) - v0;
        double df = 1.0 + 1.687 * corr;
        double vn = fmax(v - f / df, 0.0);
        if (fabs(vn - v) <= 2e-14 * fmax(1.0, fabs(v))) { v = vn; break; }
        v = vn;
    }
    double Re = fmax(K * v, 0.0), drag = 1.0 + 0.15 * pow(Re, 0.687);
    *out_Re = Re; *out_drag = drag;
    return v;
}

/* ---------------- meridional advection-diffusion field (:4040-4215, host sequence :6451-6725) ----------------
 * Sediment model 3 without a supplied grid: per size bin, the stationary axisymmetric advection-diffusion of
 * the sediment in the cell's secondary circulation on a cell-centred (r, z) grid, solved by red-black SOR
 * with mass renormalisation every 20 iterations and at every check; the solve stops at the first check
 * (after at least min(1000, max) iterations) where the largest relative residual over all bins is within
 * tolerance. Bins are independent between checks, so they run in parallel; every sum keeps its order. */
typedef struct { int FSM; double R, ZMIN, ZMEAN, DH, CORE, UPEAK; } m_geom;

/* free-surface height and slope at radius r (:4046-4057) */
static void m_surface(const m_geom* g, double r, double* zs, double* hp) {
    double rr = fmin(fmax(r, 0.0), g->R), rr2 = rr * rr, R2 = g->R * g->R;
    *zs = g->ZMEAN; *hp = 0.0;
    if (!(g->DH > 0.0) || g->FSM == 0) return;
    if (g->FSM == 1) { *zs = g->ZMEAN + g->DH * (rr2 / R2 - 0.5); *hp = 2.0 * g->DH * rr / R2; return; }
    double a2 = g->CORE * g->CORE, Hinf = g->DH * (a2 + R2) / R2;
    double hbar = Hinf * (1.0 - (a2 / R2) * log1p(R2 / a2));
    *zs = g->ZMEAN - hbar + Hinf * rr2 / (a2 + rr2);
    *hp = 2.0 * Hinf * a2 * rr / ((a2 + rr2) * (a2 + rr2));
}
/* velocity of the streamfunction psi = -2U r^2 (1 - r^2/R^2)^2 eta (1 - eta) (:4059-4073) */
static void m_velocity(const m_geom* g, double r, double z, double* ur, double* uz) {
    *ur = 0.0; *uz = 0.0;
    if (!(g->UPEAK > 0.0) || !(g->R > 0.0) || !(g->DH > 0.0) || (g->FSM == 2 && !(g->CORE > 0.0))) return;
    double rr = fmin(fmax(r, 0.0), g->R), R2 = g->R * g->R, rr2 = rr * rr, zs = g->ZMEAN, hp = 0.0;
    m_surface(g, rr, &zs, &hp);
    double H = zs - g->ZMIN;
    if (!(H > 0.0)) return;
    double eta = (z - g->ZMIN) / H;
    if (eta < 0.0) eta = 0.0;
    if (eta > 1.0) eta = 1.0;
    double sq = rr2 / R2, f = eta * (1.0 - eta), fp = 1.0 - 2.0 * eta, A = 2.0 * g->UPEAK, om = 1.0 - sq;
    *ur = A * rr * om * om * fp / H;
    *uz = -A * (2.0 * om * (1.0 - 3.0 * sq) * f - rr * om * om * fp * eta * hp / H);
}
/* radial slip of bin p interpolated from its table (:4075-4082) */
static double m_slip(const double* WR, int p, double r, double R, int NRAD) {
    if (NRAD < 2 || !(R > 0.0)) return 0.0;
    double q = fmin(fmax(r / R, 0.0), 1.0) * (double)(NRAD - 1);
    int j = (int)floor(q);
    double t = q - (double)j;
    if (j >= NRAD - 1) { j = NRAD - 2; t = 1.0; }
    const double* w = WR + (size_t)p * NRAD;
    return (1.0 - t) * w[j] + t * w[j + 1];
}
/* a point inside the liquid (:4084-4089) */
static int m_fluid(const m_geom* g, double r, double z) {
    if (z < g->ZMIN) return 0;
    double zs = g->ZMEAN, hp = 0.0;
    m_surface(g, r, &zs, &hp);
    return z < zs;
}

typedef struct {
    int NR, NZ;
    double dr, dz, target;
    const unsigned char* act;
} m_plane;

/* mass renormalisation of one bin's plane (:4176-4187); 41 when the mass is not usable */
static int m_normalize(const m_plane* P, double* G) {
    double mass = 0.0;
    for (int i = 0; i < P->NR; ++i) {
        double rw = (double)i * P->dr, re = (double)(i + 1) * P->dr, vol = 0.5 * (re * re - rw * rw) * P->dz;
        for (int k = 0; k < P->NZ; ++k) {
            int c = i * P->NZ + k;
            if (P->act[c]) mass += G[c] * vol;
        }
    }
    if (!(mass > 0.0) || !(P->target > 0.0) || !isfinite(mass)) return 41;
    double scale = P->target / mass;
    for (int c = 0; c < P->NR * P->NZ; ++c)
        if (P->act[c]) G[c] *= scale;
    return 0;
}
/* neighbour sum of cell (i, k) */
static inline double m_neigh(const m_plane* P, const double* const* A, const double* G, int i, int k, int c) {
    const int NR = P->NR, NZ = P->NZ;
    double num = 0.0;
    if (i + 1 < NR) num += A[1][c] * G[(i + 1) * NZ + k];
    if (i > 0) num += A[2][c] * G[(i - 1) * NZ + k];
    if (k + 1 < NZ) num += A[3][c] * G[i * NZ + k + 1];
    if (k > 0) num += A[4][c] * G[i * NZ + k - 1];
    return num;
}
/* one colour of the SOR sweep (:4155-4169); a colour reads only the other colour, so order is free */
static void m_relax(const m_plane* P, const double* const* A, double* G, int parity, double omega) {
    for (int i = 0; i < P->NR; ++i)
        for (int k = 0; k < P->NZ; ++k) {
            int c = i * P->NZ + k;
            if (!P->act[c] || ((i + k) & 1) != parity || !(A[0][c] > 0.0)) continue;
            double target = m_neigh(P, A, G, i, k, c) / A[0][c], old = G[c];
            double nv = (1.0 - omega) * old + omega * target;
            if (!isfinite(nv) || nv < 1e-14) nv = 1e-14;
            G[c] = nv;
        }
}
/* largest relative residual of one bin (:4184-4193) */
static double m_residual(const m_plane* P, const double* const* A, const double* G) {
    double mr = 0.0;
    for (int i = 0; i < P->NR; ++i)
        for (int k = 0; k < P->NZ; ++k) {
            int c = i * P->NZ + k;
            if (!P->act[c] || !(A[0][c] > 0.0)) continue;
            double num = m_neigh(P, A, G, i, k, c);
            double den = fmax(fabs(A[0][c] * G[c]), 1e-30), q = fabs(A[0][c] * G[c] - num) / den;
            if (q > mr) mr = q;
        }
    return mr;
}

static int meridional_solve(clo_state* S, const clr_sediment_spec* ss, const m_geom* g) {
    const int n = S->n, NR = ss->meridional_nr, NZ = ss->meridional_nz, NRAD = S->n_radial;
    const int max_it = ss->solver_max_iterations, every = ss->solver_check_interval;
    if (NR < 2 || NZ < 2 || max_it < 1 || every < 1 || !(ss->grid_zmax > g->ZMIN)) {
        snprintf(S->err, sizeof S->err, "bad meridional solver settings"); return -1;
    }
    const size_t plane = (size_t)NR * NZ;
    m_plane P = {NR, NZ, g->R / (double)NR, (ss->grid_zmax - g->ZMIN) / (double)NZ,
                 0.5 * g->R * g->R * (g->ZMEAN - g->ZMIN), NULL};
    unsigned char* act = (unsigned char*)calloc(plane, 1);
    double* G = zalloc(plane * n);
    double* coef = zalloc(5 * plane * n);
    double* res = zalloc(n);
    int* bad = (int*)calloc((size_t)n, sizeof(int));
    P.act = act;
    /* liquid cells (:4091-4098) */
    for (int i = 0; i < NR; ++i)
        for (int k = 0; k < NZ; ++k)
            act[i * NZ + k] = (unsigned char)m_fluid(g, ((double)i + 0.5) * P.dr, g->ZMIN + ((double)k + 0.5) * P.dz);
    /* the model-2 drift-diffusion field starts the iteration (:4100-4112, sediment_local_scale :1560-1593) */
    o_field F = {2, g->FSM, n, NRAD, 2, 2, S->sed_A, S->sed_B, S->sed_norm, S->sed_radial_log, NULL,
                 (float)ss->grid_zmax, (float)g->R, (float)g->ZMIN, (float)g->CORE};
    int rc = 0;
#pragma omp parallel for schedule(dynamic, 1)
    for (int p = 0; p < n; ++p) {
        double* Gp = G + (size_t)p * plane;
        double* A[5];
        for (int q = 0; q < 5; ++q) A[q] = coef + ((size_t)p * 5 + q) * plane;
        for (int i = 0; i < NR; ++i)
            for (int k = 0; k < NZ; ++k) {
                int c = i * NZ + k;
                if (!act[c]) { Gp[c] = 0.0; continue; }
                float x = (float)(((double)i + 0.5) * P.dr), z = (float)(g->ZMIN + ((double)k + 0.5) * P.dz);
                Gp[c] = o_local_scale(&F, p, x, 0.0f, z);
            }
        /* upwind finite-volume coefficients with no-flux walls (:4114-4153) */
        const double ws = S->sed_ws[p], Dt = ss->eddy_diffusivity;
        for (int i = 0; i < NR; ++i)
            for (int k = 0; k < NZ; ++k) {
                int c = i * NZ + k;
                if (!act[c]) continue;
                double rc = ((double)i + 0.5) * P.dr, zc = g->ZMIN + ((double)k + 0.5) * P.dz;
                double rw = (double)i * P.dr, re = (double)(i + 1) * P.dr, dz = P.dz, dr = P.dr;
                double Az = 0.5 * (re * re - rw * rw), ap = 0.0, ur = 0.0, uz = 0.0, V, Fl, diff;
                if (i + 1 < NR && act[(i + 1) * NZ + k] && m_fluid(g, re, zc)) {          /* east face */
                    m_velocity(g, re, zc, &ur, &uz);
                    V = ur + m_slip(S->sed_wr, p, re, g->R, NRAD); Fl = V * re * dz; diff = Dt * re * dz / dr;
                    A[1][c] = diff + fmax(-Fl, 0.0); ap += diff + fmax(Fl, 0.0);
                }
                if (i > 0 && act[(i - 1) * NZ + k] && m_fluid(g, rw, zc)) {               /* west face */
                    m_velocity(g, rw, zc, &ur, &uz);
                    V = ur + m_slip(S->sed_wr, p, rw, g->R, NRAD); Fl = -V * rw * dz; diff = Dt * rw * dz / dr;
                    A[2][c] = diff + fmax(-Fl, 0.0); ap += diff + fmax(Fl, 0.0);
                }
                double zf = zc + 0.5 * dz;
                if (k + 1 < NZ && act[i * NZ + k + 1] && m_fluid(g, rc, zf)) {           /* top face */
                    m_velocity(g, rc, zf, &ur, &uz);
                    V = uz - ws; Fl = V * Az; diff = Dt * Az / dz;
                    A[3][c] = diff + fmax(-Fl, 0.0); ap += diff + fmax(Fl, 0.0);
                }
                zf = zc - 0.5 * dz;
                if (k > 0 && act[i * NZ + k - 1] && m_fluid(g, rc, zf)) {                /* bottom face */
                    m_velocity(g, rc, zf, &ur, &uz);
                    V = uz - ws; Fl = -V * Az; diff = Dt * Az / dz;
                    A[4][c] = diff + fmax(-Fl, 0.0); ap += diff + fmax(Fl, 0.0);
                }
                A[0][c] = ap;
            }
        bad[p] = m_normalize(&P, Gp);
    }
    for (int p = 0; p < n; ++p) if (bad[p]) rc = bad[p];
    const int min_it = max_it < 1000 ? max_it : 1000;
    int iters = 0, last = 0;
    double worst = 0.0;
    for (int it0 = 0; !rc && it0 < max_it;) {
        /* the next check: a multiple of the interval, or the last iteration */
        int it1 = (it0 / every + 1) * every;
        if (it1 > max_it) it1 = max_it;
#pragma omp parallel for schedule(dynamic, 1)
        for (int p = 0; p < n; ++p) {
            double* Gp = G + (size_t)p * plane;
            const double* A[5];
            for (int q = 0; q < 5; ++q) A[q] = coef + ((size_t)p * 5 + q) * plane;
            for (int it = it0 + 1; it <= it1; ++it) {
                m_relax(&P, A, Gp, 0, ss->solver_sor);
                m_relax(&P, A, Gp, 1, ss->solver_sor);
                if (it % 20 == 0 && m_normalize(&P, Gp)) bad[p] = 41;
            }
            if (m_normalize(&P, Gp)) bad[p] = 41;
            res[p] = m_residual(&P, A, Gp);
        }
        for (int p = 0; p < n; ++p) if (bad[p]) rc = bad[p];
        if (rc) break;
        last = it1;
        worst = 0.0;
        for (int p = 0; p < n; ++p) worst = res[p] > worst ? res[p] : worst;
        if (it1 >= min_it && worst <= ss->solver_tolerance) { iters = it1; break; }
        it0 = it1;
    }
    if (iters == 0) iters = last ? last : max_it;
    S->solver_iterations = iters;
    S->solver_residual = worst;
    if (!rc && worst > ss->solver_tolerance) rc = -7;
    if (!rc) {
        /* extend every column above the free surface with its highest liquid value (:4195-4201) */
        for (int p = 0; p < n; ++p)
            for (int i = 0; i < NR; ++i) {
                double* col = G + (size_t)p * plane + (size_t)i * NZ;
                int top = -1;
                for (int k = NZ - 1; k >= 0; --k)
                    if (act[i * NZ + k]) { top = k; break; }
                if (top < 0) { for (int k = 0; k < NZ; ++k) col[k] = 1.0; continue; }
                for (int k = top + 1; k < NZ; ++k) col[k] = col[top];
            }
        /* finalisation and majorants (:4203-4220) */
        double mg = 0.0, mw = 0.0;
        for (int p = 0; p < n; ++p) {
            double mx = 0.0;
            for (size_t c = 0; c < plane; ++c)
                if (act[c] && G[(size_t)p * plane + c] > mx) mx = G[(size_t)p * plane + c];
            if (!(mx > 0.0)) mx = 1.0;
            S->sed_norm[p] = 1.0;
            S->sed_max[p] = mx;
        }
        for (int i = 0; i < n; ++i) { mg += S->trace_geom[i] * S->sed_max[i]; mw += S->trace_wave[i] * S->sed_max[i]; }
        S->sed_major[0] = mg; S->sed_major[1] = mw; S->sed_major[2] = mg + mw;
        free(S->sed_grid);
        S->sed_grid = G;
        G = NULL;
        S->grid_nr = NR; S->grid_nz = NZ;
    } else if (rc == -7) {
        snprintf(S->err, sizeof S->err, "meridional transport solver did not converge");
    } else {
        snprintf(S->err, sizeof S->err, "meridional normalization error %d", rc);
    }
    free(act); free(G); free(coef); free(res); free(bad);
    return rc;
}

int clo_prepare(const clr_scene_params* sp, const clr_particle_spec* ps, const clr_sediment_spec* ss, clo_state** out) {
    if (!sp || !ps || !ss || !out) return -1;
    clo_state* S = (clo_state*)calloc(1, sizeof(clo_state));
    *out = S;
    S->sp = *sp;
    const int n = ps->n_bins;
    S->n = n;
    if (n < 1 || n > CLR_MAX_BINS) { snprintf(S->err, sizeof S->err, "bad n_bins %d", n); return -1; }
    S->d = zalloc(n); S->wd = zalloc(n); S->nidx = zalloc(n); S->kidx = zalloc(n);
    double sw = 0.0;
    for (int i = 0; i < n; ++i) {
        S->d[i] = ps->diameter_m[i]; S->nidx[i] = ps->n_real[i]; S->kidx[i] = ps->k_imag[i];
        sw += ps->weight[i];
    }
    /* PSD normalisation: the aggregation kernel with zero exposure (:3607-3635) */
    if (!(ps->density_kg_m3 > 0.0) || ps->concentration_kg_m3 < 0.0) { snprintf(S->err, sizeof S->err, "bad density/concentration"); return 21; }
    if (!(sw > 0.0)) { snprintf(S->err, sizeof S->err, "weights sum to zero"); return 22; }
    for (int i = 0; i < n; ++i) S->wd[i] = ps->weight[i] / sw;
    /* Mie (:3495-3559) */
    cd_t* D = (cd_t*)calloc(CLR_MIE_MAX_ORDER + 1, sizeof(cd_t));
    cd_t* A = (cd_t*)calloc((size_t)n * CLR_MIE_MAX_ORDER, sizeof(cd_t));
    cd_t* B = (cd_t*)calloc((size_t)n * CLR_MIE_MAX_ORDER, sizeof(cd_t));
    S->nstop = (int*)calloc(n, sizeof(int));
    S->x = zalloc(n); S->qext = zalloc(n); S->qsca = zalloc(n); S->qabs = zalloc(n); S->qback = zalloc(n);
    S->g = zalloc(n); S->albedo = zalloc(n);
    int err = 0;
    for (int p = 0; p < n; ++p) {
        int e = mie_bin(S->d[p], S->nidx[p], S->kidx[p], ps->n_medium, ps->wavelength_m, D, A + (size_t)p * CLR_MIE_MAX_ORDER,
                        B + (size_t)p * CLR_MIE_MAX_ORDER, &S->nstop[p], &S->x[p], &S->qext[p], &S->qsca[p], &S->qabs[p],
                        &S->qback[p], &S->g[p], &S->albedo[p]);
        if (e) err = e;
    }
    free(D);
    if (err) { free(A); free(B); snprintf(S->err, sizeof S->err, "Mie precompute error %d", err); return err; }
    const int em = sp->event_model;
    if (em == 3 || em == 4 || em == 5) {
        const int nt = ps->n_theta;
        S->nt = nt;
        S->theta = zalloc(nt);
        S->phase_cdf = zalloc((size_t)n * nt);
        for (int j = 0; j < nt; ++j) {
            if (j == 0) S->theta[j] = 0.0;
            else if (j == nt - 1) S->theta[j] = O_PI_D;
            else { double u = (double)j / (double)(nt - 1); S->theta[j] = 0.5 * O_PI_D * (1.0 - cos(O_PI_D * u)); }
        }
        double* pdf = zalloc((size_t)n * nt);
#pragma omp parallel for schedule(static)
        for (long long idx = 0; idx < (long long)n * nt; ++idx) {
            int p = (int)(idx / nt), j = (int)(idx - (long long)p * nt);
            pdf[idx] = mie_pdf(S->theta[j], S->nstop[p], A + (size_t)p * CLR_MIE_MAX_ORDER, B + (size_t)p * CLR_MIE_MAX_ORDER);
        }
        /* trapezoid CDF, normalise, force monotone (:3583-3592) */
        for (int p = 0; p < n; ++p) {
            double* cdf = S->phase_cdf + (size_t)p * nt;
            const double* pd = pdf + (size_t)p * nt;
            cdf[0] = 0.0;
            double s = 0.0;
            for (int j = 1; j < nt; ++j) {
                double area = 0.5 * (pd[j] + pd[j - 1]) * (S->theta[j] - S->theta[j - 1]);
                if (area < 0.0 && area > -1e-18) area = 0.0;
                s += area;
                cdf[j] = s;
            }
            if (!(s > 0.0) || !isfinite(s)) {
                err = 3;
                for (int j = 0; j < nt; ++j) cdf[j] = (double)j / (double)(nt - 1);
                continue;
            }
            double prev = 0.0;
            for (int j = 0; j < nt; ++j) {
                double v = cdf[j] / s;
                if (v < prev) v = prev;
                if (v > 1.0) v = 1.0;
                cdf[j] = v;
                prev = v;
            }
            cdf[nt - 1] = 1.0;
        }
        free(pdf);
    } else {
        S->nt = 2;
        S->theta = zalloc(2);
        S->phase_cdf = zalloc((size_t)2 * n);
        S->theta[0] = 0.0; S->theta[1] = O_PI_D;
        for (int p = 0; p < n; ++p) { S->phase_cdf[2 * p] = 0.0; S->phase_cdf[2 * p + 1] = 1.0; }
    }
    free(A); free(B);
    if (err) { snprintf(S->err, sizeof S->err, "phase CDF error"); return err; }
    /* transport rates and channel CDFs (:3845-3921) */
    S->radius = zalloc(n); S->nden = zalloc(n); S->mug = zalloc(n); S->mus = zalloc(n); S->mue = zalloc(n);
    S->muw = zalloc(n); S->muev = zalloc(n); S->gcdf = zalloc(n); S->wcdf = zalloc(n); S->pcdf = zalloc(n);
    S->muscal = zalloc(8);
    {
        double* pmass = zalloc(n); double* srcw = zalloc(n);
        double *sgv = zalloc(n), *ssv = zalloc(n), *sev = zalloc(n), *swv = zalloc(n);
        double sw2 = 0.0;
        for (int i = 0; i < n; ++i) sw2 += S->wd[i];
        if (!(sw2 > 0.0)) err = 4;
        double avg_mass = 0.0;
        for (int i = 0; i < n && !err; ++i) {
            double r = 0.5 * S->d[i];
            S->radius[i] = r;
            srcw[i] = S->wd[i] / sw2;
            double m = ps->density_kg_m3 * (4.0 / 3.0) * O_PI_D * r * r * r;
            pmass[i] = m;
            avg_mass += srcw[i] * m;
        }
        for (int i = 0; i < n && !err; ++i) {
            double nd = 0.0;
            if (ps->weight_mode == 0) nd = ps->concentration_kg_m3 * srcw[i] / pmass[i];
            else nd = (avg_mass > 0.0 ? ps->concentration_kg_m3 / avg_mass : 0.0) * srcw[i];
            S->nden[i] = nd;
            double sg = O_PI_D * S->radius[i] * S->radius[i], sa = fmax(S->qsca[i], 0.0) * sg, se = fmax(S->qext[i], 0.0) * sg;
            double tol = 1e-10 * fmax(1.0, fmax(fabs(S->qext[i]), fabs(S->qsca[i])));
            const double ki = S->kidx[i];
            if (!isfinite(ki) || ki < 0.0 || !isfinite(S->qext[i]) || !isfinite(S->qsca[i]) || S->qext[i] < -tol ||
                S->qsca[i] < -tol || S->qsca[i] > S->qext[i] + tol || (ki == 0.0 && fabs(S->qext[i] - S->qsca[i]) > tol)) {
                err = 5;
                break;
            }
            double sw_ = 0.0;
            if (em == 3) sw_ = ps->hybrid_wave_scale * fmax(S->qsca[i] - 1.0, 0.0) * sg;
            else if (em == 4 || em == 5) {
                double rate = (ki > 0.0) ? se : sa;
                sw_ = (ki > 0.0) ? ((sa > 0.0) ? rate * fmax(sa - sg, 0.0) / sa : 0.0) : fmax(sa - sg, 0.0);
            }
            sgv[i] = sg; ssv[i] = sa; sev[i] = se; swv[i] = sw_;
            S->mug[i] = nd * sg; S->mus[i] = nd * sa; S->mue[i] = nd * se; S->muw[i] = nd * sw_;
        }
        if (!err) {
            double mg = 0.0, ms = 0.0, me = 0.0, mw = 0.0;
            for (int i = 0; i < n; ++i) { mg += S->mug[i]; ms += S->mus[i]; me += S->mue[i]; mw += S->muw[i]; }
            double mt = 0.0;
            for (int i = 0; i < n; ++i) {
                double mb;
                if (em == 0) mb = S->mug[i];
                else if (em == 1) mb = S->mus[i];
                else if (em == 2) mb = S->mue[i];
                else if (em == 3) mb = S->mug[i] + S->muw[i];
                else mb = (S->kidx[i] > 0.0) ? S->mue[i] : S->mus[i];
                S->muev[i] = mb;
                mt += mb;
            }
            int hyb = (em == 3) || (em == 4) || (em == 5);
            double mtrace_geom = ((em == 4) || (em == 5)) ? fmax(mt - mw, 0.0) : ((em == 3) ? mg : mt);
            double mtrace_wave = hyb ? mw : 0.0;
            double cg = 0.0, cw = 0.0, ct = 0.0;
            for (int i = 0; i < n; ++i) {
                double mgi = ((em == 4) || (em == 5)) ? fmax(S->muev[i] - S->muw[i], 0.0) : S->mug[i];
                double pg = hyb ? (mtrace_geom > 0.0 ? mgi / mtrace_geom : 0.0) : (mt > 0.0 ? S->muev[i] / mt : 0.0);
                double pw = (hyb && mtrace_wave > 0.0 ? S->muw[i] / mtrace_wave : 0.0), pt = (mt > 0.0 ? S->muev[i] / mt : 0.0);
                cg += pg; cw += pw; ct += pt;
                S->gcdf[i] = cg; S->wcdf[i] = cw; S->pcdf[i] = ct;
            }
            if (n > 0) {
                if (cg > 0.0) S->gcdf[n - 1] = 1.0;
                if (cw > 0.0) S->wcdf[n - 1] = 1.0;
                if (ct > 0.0) S->pcdf[n - 1] = 1.0;
            }
            S->muscal[0] = mtrace_geom; S->muscal[1] = mtrace_wave; S->muscal[2] = mg; S->muscal[3] = ms;
            S->muscal[4] = me; S->muscal[5] = mtrace_wave; S->muscal[6] = mt;
            double cwave = 1.0;
            if (hyb && ps->wave_rms_height_m > 0.0 && ps->wavelength_m > 0.0 && ps->n_medium > 0.0) {
                double a = 4.0 * O_PI_D * ps->n_medium * ps->wave_rms_height_m / ps->wavelength_m;
                cwave = exp(-a * a);
                if (cwave < 0.0) cwave = 0.0;
                if (cwave > 1.0) cwave = 1.0;
            }
            S->muscal[7] = cwave;
        }
        free(pmass); free(srcw); free(sgv); free(ssv); free(sev); free(swv);
    }
    if (err) { snprintf(S->err, sizeof S->err, "transport precompute error %d", err); return err; }
    S->moment_a = zalloc(n); S->moment_b = zalloc(n);
    S->moment_mode = (unsigned char*)calloc(n, 1);
    for (int i = 0; i < n; ++i) {
        S->moment_a[i] = 1.0;
        if (ps->moment_enabled && ps->moment_a && ps->moment_b && ps->moment_mode) {
            S->moment_a[i] = ps->moment_a[i]; S->moment_b[i] = ps->moment_b[i]; S->moment_mode[i] = ps->moment_mode[i];
        }
    }
    /* channel rates traced by the hybrid laws (:6362-6375) */
    S->trace_geom = zalloc(n); S->trace_wave = zalloc(n);
    for (int i = 0; i < n; ++i) {
        if (em == 3) { S->trace_geom[i] = S->mug[i]; S->trace_wave[i] = S->muw[i]; }
        else if (em == 4 || em == 5) { S->trace_geom[i] = fmax(S->muev[i] - S->muw[i], 0.0); S->trace_wave[i] = S->muw[i]; }
        else { S->trace_geom[i] = S->muev[i]; S->trace_wave[i] = 0.0; }
    }
    /* sediment coefficients and majorants (:3940-4038) */
    const int NRAD = ss->n_radial;
    S->n_radial = NRAD;
    S->sed_A = zalloc(n); S->sed_B = zalloc(n); S->sed_norm = zalloc(n); S->sed_max = zalloc(n);
    S->sed_radial_log = zalloc((size_t)n * NRAD); S->sed_major = zalloc(4);
    S->sed_ws = zalloc(n); S->sed_wr = zalloc((size_t)n * NRAD);
    const int TM = sp->sediment_model, FSM = sp->free_surface_model;
    /* FP64 geometry as the reference passes it (float64 arguments, CLARITAS/CLARITAS.py:6413-6418);
       a spec without it widens the scene's FP32 values */
    const int g64 = ss->rin > 0.0;
    const double R = g64 ? ss->rin : (double)sp->rin, ZMIN = g64 ? ss->zmin : (double)sp->zmin;
    const double ZMEAN = g64 ? ss->zmean : (double)sp->zmean;
    const double DH = g64 ? ss->vortex_delta_h : (double)sp->vortex_delta_h;
    const double CORE = g64 ? ss->vortex_core_radius : (double)sp->vortex_core_radius;
    if (TM == 0) {
        double mg = 0.0, mw = 0.0;
        for (int i = 0; i < n; ++i) { S->sed_norm[i] = 1.0; S->sed_max[i] = 1.0; mg += S->trace_geom[i]; mw += S->trace_wave[i]; }
        S->sed_major[0] = mg; S->sed_major[1] = mw; S->sed_major[2] = mg + mw; S->sed_major[3] = 0.0;
    } else {
        const double rho_p = ss->particle_density, rho_w = ss->water_density, mu = ss->water_viscosity;
        const double grav = ss->gravity, Dt = ss->eddy_diffusivity;
        const int NQ = ss->n_quad;
        if ((TM != 1 && TM != 2 && TM != 3) || !(rho_p > rho_w) || !(rho_w > 0.0) || !(mu > 0.0) || !(grav > 0.0) ||
            !(Dt > 0.0) || !(R > 0.0) || NQ < 64 || NRAD < 65) {
            snprintf(S->err, sizeof S->err, "sediment precompute error 31"); return 31;
        }
        /* surface model 3 (the Rankine vortex, new) is accepted with a supplied model-3 field only */
        if (FSM < 0 || FSM > 3 || (FSM == 3 && TM != 3) || (DH > 0.0 && FSM == 0) || (FSM >= 2 && !(CORE > 0.0))) {
            snprintf(S->err, sizeof S->err, "sediment precompute error 32"); return 32;
        }
        double R2 = R * R, a2 = CORE * CORE, Hinf = 0.0, hbar = 0.0, omega2 = 0.0;
        if (DH > 0.0 && FSM == 1) { Hinf = DH; hbar = 0.5 * DH; omega2 = 2.0 * grav * DH / R2; }
        else if (DH > 0.0 && FSM == 2) {
            Hinf = DH * (a2 + R2) / R2; hbar = Hinf * (1.0 - (a2 / R2) * log1p(R2 / a2)); omega2 = 2.0 * grav * Hinf / a2;
        }
        double fR = (FSM == 2) ? R2 / (a2 + R2) : R2;
        double Hmean = ZMEAN - ZMIN, dr = R / (double)NQ, drad = R / (double)(NRAD - 1);
        if (!(Hmean > 0.0)) { snprintf(S->err, sizeof S->err, "sediment precompute error 33"); return 33; }
        double major_g = 0.0, major_w = 0.0, maxAeq = 0.0;
        double* wr_arr = zalloc(NRAD);
        for (int i = 0; i < n; ++i) {
            double d = S->d[i];
            double tau = rho_p * d * d / (18.0 * mu);
            double ws0 = (rho_p - rho_w) * grav * d * d / (18.0 * mu);
            double sre = 0.0, sdrag = 1.0;
            double ws = (TM == 2 || TM == 3) ? schiller_naumann(ws0, d, rho_w, mu, &sre, &sdrag) : ws0;
            double Bc = ws / Dt;
            S->sed_B[i] = Bc;
            S->sed_ws[i] = ws;
            long long base = (long long)i * NRAD;
            double* RL = S->sed_radial_log + base;
            if (TM == 1) {
                double Ac = tau * omega2 * ((FSM == 2) ? a2 : 1.0) / (2.0 * Dt);
                S->sed_A[i] = Ac;
                if (Ac > maxAeq) maxAeq = Ac;
                for (int j = 0; j < NRAD; ++j) {
                    double r = (double)j * drad, rr2 = r * r, f = (FSM == 2) ? rr2 / (a2 + rr2) : rr2;
                    RL[j] = Ac * (f - fR);
                }
            } else {
                double total = 0.0, prev = 0.0;
                for (int j = 0; j < NRAD; ++j) {
                    double r = (double)j * drad, acc = 0.0;
                    if (r > 0.0) acc = (FSM == 1) ? omega2 * r : ((FSM == 2) ? omega2 * r / pow(1.0 + r * r / a2, 2.0) : 0.0);
                    double w0 = tau * acc, re = 0.0, drag = 1.0;
                    double wr = schiller_naumann(w0, d, rho_w, mu, &re, &drag);
                    wr_arr[j] = wr;
                    S->sed_wr[base + j] = wr;
                    if (j > 0) total += 0.5 * (prev + wr) * drad;
                    prev = wr;
                }
                double cum = 0.0;
                prev = 0.0;
                for (int j = 0; j < NRAD; ++j) {
                    double wr = wr_arr[j];
                    if (j > 0) cum += 0.5 * (prev + wr) * drad;
                    prev = wr;
                    double psi = (cum - total) / Dt;
                    if (psi > 0.0) psi = 0.0;
                    RL[j] = psi;
                }
                RL[NRAD - 1] = 0.0;
                double Aeq = (fR > 0.0) ? -RL[0] / fR : 0.0;
                S->sed_A[i] = Aeq;
                if (Aeq > maxAeq) maxAeq = Aeq;
            }
            double integ = 0.0;
            for (int j = 0; j < NQ; ++j) {
                double r = ((double)j + 0.5) * dr, rr2 = r * r;
                double zsurf = ZMEAN;
                if (FSM == 1 && DH > 0.0) zsurf = ZMEAN + DH * (rr2 / R2 - 0.5);
                else if (FSM == 2 && DH > 0.0) zsurf = ZMEAN - hbar + Hinf * rr2 / (a2 + rr2);
                double Hh = fmax(zsurf - ZMIN, 0.0);
                double radial_log;
                if (TM == 1) {
                    double f = (FSM == 2) ? rr2 / (a2 + rr2) : rr2;
                    radial_log = S->sed_A[i] * (f - fR);
                } else {
                    double u = r / R * (double)(NRAD - 1);
                    int k = (int)floor(u);
                    if (k < 0) k = 0;
                    if (k > NRAD - 2) k = NRAD - 2;
                    double t = u - (double)k;
                    radial_log = (1.0 - t) * RL[k] + t * RL[k + 1];
                    if (radial_log > 0.0) radial_log = 0.0;
                }
                double radial = exp(radial_log);
                double iz = (fabs(Bc) < 1e-14) ? radial * Hh : radial * (-expm1(-Bc * Hh)) / Bc;
                integ += r * iz;
            }
            double norm = (2.0 / (R2 * Hmean)) * integ * dr;
            if (!(norm > 0.0) || !isfinite(norm)) { free(wr_arr); snprintf(S->err, sizeof S->err, "sediment precompute error 34"); return 34; }
            double mx = 1.0 / norm;
            S->sed_norm[i] = norm;
            S->sed_max[i] = mx;
            major_g += S->trace_geom[i] * mx;
            major_w += S->trace_wave[i] * mx;
        }
        free(wr_arr);
        S->sed_major[0] = major_g; S->sed_major[1] = major_w; S->sed_major[2] = major_g + major_w; S->sed_major[3] = maxAeq;
        if (!(S->sed_major[2] >= 0.0) || !isfinite(S->sed_major[2])) { snprintf(S->err, sizeof S->err, "sediment precompute error 35"); return 35; }
    }
    S->grid_nr = 2; S->grid_nz = 2; S->grid_zmax = (float)ss->grid_zmax;
    S->sed_grid = zalloc(1);
    S->sed_grid[0] = 1.0;
    if (TM == 3 && !ss->grid) {
        m_geom g = {FSM, R, ZMIN, ZMEAN, DH, CORE, ss->meridional_peak_speed};
        int rc = meridional_solve(S, ss, &g);
        if (rc) return rc;
    } else if (TM == 3) {
        /* caller-supplied grid, every cell active: finalisation + majorants (:4203-4220) */
        if (!ss->grid || ss->grid_nr < 2 || ss->grid_nz < 2) { snprintf(S->err, sizeof S->err, "model 3 needs a grid"); return -1; }
        S->grid_nr = ss->grid_nr; S->grid_nz = ss->grid_nz;
        size_t plane = (size_t)ss->grid_nr * ss->grid_nz;
        free(S->sed_grid);
        S->sed_grid = zalloc(plane * n);
        memcpy(S->sed_grid, ss->grid, plane * n * sizeof(double));
        double mg = 0.0, mw = 0.0;
        for (int p = 0; p < n; ++p) {
            double mx = 0.0;
            for (size_t c = 0; c < plane; ++c) { double q = S->sed_grid[(size_t)p * plane + c]; if (q > mx) mx = q; }
            if (!(mx > 0.0)) mx = 1.0;
            S->sed_norm[p] = 1.0;
            S->sed_max[p] = mx;
        }
        for (int i = 0; i < n; ++i) { mg += S->trace_geom[i] * S->sed_max[i]; mw += S->trace_wave[i] * S->sed_max[i]; }
        S->sed_major[0] = mg; S->sed_major[1] = mw; S->sed_major[2] = mg + mw;
    }
    return 0;
}

int clo_n_theta(clo_state* s) { return s ? s->nt : 0; }

int clo_read_sediment(clo_state* S, double* A, double* B, double* norm, double* ws, double* radial_log,
                      double* radial_slip) {
    if (!S || !S->sed_A) return -1;
    const size_t n = (size_t)S->n, nr = (size_t)S->n_radial;
    if (A) memcpy(A, S->sed_A, n * sizeof(double));
    if (B) memcpy(B, S->sed_B, n * sizeof(double));
    if (norm) memcpy(norm, S->sed_norm, n * sizeof(double));
    if (ws) memcpy(ws, S->sed_ws, n * sizeof(double));
    if (radial_log) memcpy(radial_log, S->sed_radial_log, n * nr * sizeof(double));
    if (radial_slip) memcpy(radial_slip, S->sed_wr, n * nr * sizeof(double));
    return 0;
}

double clo_meridional_velocity(int fsm, double r, double z, double zmin, double zmean, double R, double dh, double core,
                               double upeak, double* uz) {
    m_geom g = {fsm, R, zmin, zmean, dh, core, upeak};
    double ur = 0.0, w = 0.0;
    m_velocity(&g, r, z, &ur, &w);
    if (uz) *uz = w;
    return ur;
}

float clo_surface(int fsm, float x, float y, float zmean, float R, float dh, float core, float* normal) {
    if (normal) o_surface_normal(x, y, R, fsm, dh, core, normal, normal + 1, normal + 2);
    return o_surface_z(x, y, zmean, R, fsm, dh, core);
}

float clo_surface_hit(int fsm, float x, float y, float z, float vx, float vy, float vz, float zmean, float R, float dh,
                      float core) {
    return o_surface_hit(x, y, z, vx, vy, vz, zmean, R, fsm, dh, core);
}

double clo_local_scale(clo_state* S, int pidx, float x, float y, float z) {
    if (!S || pidx < 0 || pidx >= S->n) return -1.0;
    const clr_scene_params* P = &S->sp;
    o_field F = {P->sediment_model, P->free_surface_model, S->n, S->n_radial, S->grid_nr, S->grid_nz, S->sed_A, S->sed_B,
                 S->sed_norm, S->sed_radial_log, S->sed_grid, S->grid_zmax, P->rin, P->zmin, P->vortex_core_radius};
    return o_local_scale(&F, pidx, x, y, z);
}

int clo_meridional_fluid(int fsm, double r, double z, double zmin, double zmean, double R, double dh, double core) {
    m_geom g = {fsm, R, zmin, zmean, dh, core, 0.0};
    return m_fluid(&g, r, z);
}

int clo_read_sediment_field(clo_state* S, double* grid, int* nr, int* nz, int* iterations, double* max_residual) {
    if (!S) return -1;
    if (nr) *nr = S->grid_nr;
    if (nz) *nz = S->grid_nz;
    if (iterations) *iterations = S->solver_iterations;
    if (max_residual) *max_residual = S->solver_residual;
    if (grid) memcpy(grid, S->sed_grid, (size_t)S->n * S->grid_nr * S->grid_nz * sizeof(double));
    return 0;
}

int clo_read_physics(clo_state* S, clr_particle_physics* o) {
    if (!S || !o) return -1;
    const int n = S->n;
#define CP(dst, src, cnt) do { if (dst) memcpy(dst, src, (size_t)(cnt) * sizeof(double)); } while (0)
    CP(o->size_parameter, S->x, n); CP(o->qext, S->qext, n); CP(o->qsca, S->qsca, n); CP(o->qabs, S->qabs, n);
    CP(o->qback, S->qback, n); CP(o->asym_g, S->g, n); CP(o->albedo, S->albedo, n);
    if (o->nstop) memcpy(o->nstop, S->nstop, n * sizeof(int));
    CP(o->radius, S->radius, n); CP(o->number_density, S->nden, n);
    CP(o->mu_geom_bin, S->mug, n); CP(o->mu_sca_bin, S->mus, n); CP(o->mu_ext_bin, S->mue, n);
    CP(o->mu_wave_bin, S->muw, n); CP(o->mu_event_bin, S->muev, n);
    CP(o->trace_geom_bin, S->trace_geom, n); CP(o->trace_wave_bin, S->trace_wave, n);
    CP(o->geometric_cdf, S->gcdf, n); CP(o->wave_cdf, S->wcdf, n); CP(o->particle_event_cdf, S->pcdf, n);
    CP(o->mu_scalars, S->muscal, 8); CP(o->sed_majorants, S->sed_major, 4);
    CP(o->theta, S->theta, S->nt); CP(o->phase_cdf, S->phase_cdf, (size_t)n * S->nt);
#undef CP
    return 0;
}

/* ---------------- conditional closure for absorbing bins (:4479-4536) ---------------- */
typedef struct {
    float x, y, z, vx, vy, vz, path;
    o_pcount pc;
    int status, channel, event_type, macro, micro, failure, subcode;
} o_hist;

static o_hist o_conditional(uint32_t* s, int pidx, double qs, double qe, float nm, float nr, float ki, float wl,
                            float rough, float radius, float aspect, int orientation, float kappa, int max_bounces,
                            float coherent, const double* cdf, const double* theta, int nt, float x, float y, float z,
                            float vx, float vy, float vz, float rin, float zmin, float zmean, int surface, float delta,
                            float core, int max_trials, unsigned long long* stats) {
    o_hist h;
    memset(&h, 0, sizeof h);
    h.failure = OP_OTHER; h.subcode = 9002;
    double tol = 1e-10 * fmax(1.0, fmax(fabs(qs), fabs(qe)));
    if (max_trials == 0) { h.subcode = 9001; ++stats[9]; return h; }
    if (!isfinite(qs) || !isfinite(qe) || qe <= 0.0 || qs < -tol || qs > qe + tol || max_trials < 1) { ++stats[8]; return h; }
    double albedo = (ki == 0.0f && fabs(qe - qs) <= tol) ? 1.0 : fmin(fmax(qs / qe, 0.0), 1.0);
    double pabs = (ki == 0.0f && fabs(qe - qs) <= tol) ? 0.0 : fmin(fmax((qe - qs) / qe, 0.0), 1.0);
    const double MINP = 2.3283064365386962890625e-10;
    if ((ki > 0.0f && (pabs <= 0.0 || albedo >= 1.0)) || (albedo > 0.0 && albedo < MINP) || (pabs > 0.0 && pabs < MINP)) {
        h.subcode = 9003; ++stats[8]; return h;
    }
    int target_absorbed = (albedo < 1.0 && o_uniform53(s) >= albedo);
    double wave = qs > 0.0 ? fmax(qs - 1.0, 0.0) / qs : 0.0;
    for (int trial = 0; trial < max_trials; ++trial) {
        ++stats[0];
        memset(&h, 0, sizeof h);
        h.x = x; h.y = y; h.z = z; h.vx = vx; h.vy = vy; h.vz = vz;
        h.channel = (o_uniform53(s) < wave) ? ((coherent >= 1.0f || o_uniform53(s) < coherent) ? 1 : 2) : 0;
        if (h.channel == 1) {
            o_mie_direction(s, cdf, theta, nt, pidx, &h.vx, &h.vy, &h.vz);
            h.status = 1; h.event_type = 4;
        } else if (h.channel == 2) {
            float fr = sqrtf(x * x + y * y), fx = 1, fy = 0;
            if (fr > 1e-12f) { fx = -y / fr; fy = x / fr; }
            h.status = o_spheroid_event(s, nm, nr, ki, wl, rough, radius, aspect, orientation, kappa, fx, fy, 0,
                                        max_bounces, &h.vx, &h.vy, &h.vz, &h.path, &h.pc, &h.failure, &h.subcode,
                                        &h.macro, &h.micro);
            h.event_type = h.pc.entry_reflections ? 5 : (h.pc.internal_reflections ? 7 : 6);
        } else {
            float rho, phi, gx, gy, gz;
            o_sphere_geometry(s, radius, x, y, z, vx, vy, vz, &rho, &phi, &gx, &gy, &gz);
            double dcx = (double)x - (double)radius * gx, dcy = (double)y - (double)radius * gy,
                   dcz = (double)z - (double)radius * gz;
            if (!o_sphere_accessible(dcx, dcy, dcz, radius, rin, zmin, zmean, surface, delta, core)) { ++stats[2]; continue; }
            h.status = o_sphere_sampled(s, nm, nr, ki, wl, rough, radius, max_bounces, gx, gy, gz, dcx, dcy, dcz, &h.x,
                                        &h.y, &h.z, &h.vx, &h.vy, &h.vz, &h.path, &h.pc, &h.failure, &h.subcode,
                                        &h.macro, &h.micro);
            h.event_type = h.pc.entry_reflections ? 1 : (h.pc.internal_reflections ? 3 : 2);
        }
        if (h.status != 1 && h.status != 2) { ++stats[8]; return h; }
        if ((h.status == 2) != target_absorbed) { ++stats[1]; continue; }
        ++stats[3 + h.channel];
        ++stats[h.status == 2 ? 6 : 7];
        return h;
    }
    memset(&h, 0, sizeof h);
    h.failure = OP_OTHER; h.subcode = 9001;
    ++stats[9];
    return h;
}

/* Mie two-moment post-outcome angular map (:4459-4476) */
static void o_moment(float vinx, float viny, float vinz, float* vx, float* vy, float* vz, float A, float B) {
    float c = fminf(fmaxf(o_dot(vinx, viny, vinz, *vx, *vy, *vz), -1.0f), 1.0f);
    float d = fminf(fmaxf(1.0f - c, 0.0f), 2.0f);
    float dm = fminf(fmaxf(A * d + B * d * d, 0.0f), 2.0f);
    float cp = 1.0f - dm;
    float px = *vx - c * vinx, py = *vy - c * viny, pz = *vz - c * vinz;
    float pn = sqrtf(fmaxf(px * px + py * py + pz * pz, 0.0f));
    if (pn > 1.0e-8f) { px /= pn; py /= pn; pz /= pn; }
    else {
        float e1x, e1y, e1z, e2x, e2y, e2z;
        o_perp_basis(vinx, viny, vinz, &e1x, &e1y, &e1z, &e2x, &e2y, &e2z);
        px = e1x; py = e1y; pz = e1z;
    }
    float sp = sqrtf(fmaxf(1.0f - cp * cp, 0.0f));
    *vx = cp * vinx + sp * px; *vy = cp * viny + sp * py; *vz = cp * vinz + sp * pz;
    o_normalize(vx, vy, vz);
}

/* ---------------- one photon history (:4608-5103) ---------------- */
typedef struct {
    int ic, gic, wic, wcoh, wmorph, cir, cor, ctir, tr, ttir, bir, bor, btir, sbi, sbr, entered, st, pf, pfs;
    o_pcount pc;
    int steps, nulls;
    float wp, ap, ax, ay, az, avx, avy, avz;
    /* particle-event provenance (:4625-4633): first/last event type and order, first-event backscatter and
       source hemisphere, first/last particle, geometric and wave bin, acrylic returns after a particle
       event and particle events after such a return, first/last deflection */
    int first_evt, last_evt, last_order, first_back, first_hemi, bins[6], acr_returns, after_return;
    float first_defl, last_defl;
    /* path inside particles and its optical length over all events, water path at the last event (:4633) */
    float ipath_total, iopl_total, wp_last;
} o_ray;

/* The bins and types of a particle event of type `type` in bin `pidx` (:4836-4848 for an absorbed
   conditional encounter, :4972-4978 for a survived event). */
static void o_prov_mark(o_ray* r, int type, int pidx) {
    if (r->bins[0] < 0) r->bins[0] = pidx;
    r->bins[1] = pidx;
    if (type >= 1 && type <= 3) { if (r->bins[2] < 0) r->bins[2] = pidx; r->bins[3] = pidx; }
    else if (type >= 4 && type <= 7) { if (r->bins[4] < 0) r->bins[4] = pidx; r->bins[5] = pidx; }
    if (r->acr_returns > 0) r->after_return++;
    if (r->ic == 1) r->first_evt = type;
    r->last_evt = type;
    r->last_order = r->ic;
}

static void o_trace_ray(const clo_state* S, uint32_t gid, uint32_t seed0, uint32_t seed1, uint32_t seed2,
                        unsigned long long* cstats, o_ray* out) {
    const clr_scene_params* P = &S->sp;
    o_ray r;
    memset(&r, 0, sizeof r);
    r.ax = r.ay = r.az = r.avx = r.avy = r.avz = NAN;
    for (int k = 0; k < 6; ++k) r.bins[k] = -1;
    r.first_defl = r.last_defl = -1.0f;
    r.wp_last = -1.0f;
    uint32_t state = seed0 + gid * 74729u + 13u, stOPT = seed1 + gid * 104729u + 29u, stSRC = seed2 + gid * 130363u + 43u;
    const int TM = P->sediment_model, FSM = P->free_surface_model;
    const float RIN = P->rin, ZMIN = P->zmin, ZMEAN = P->zmean, ZTOP = P->zwall_top, DH = P->vortex_delta_h,
                CORE = P->vortex_core_radius;
    const float MU_GEOM = (float)S->muscal[0], MU_WAVE = (float)S->muscal[1];
    const float MU_MAJOR_GEOM = (TM == 0) ? MU_GEOM : (float)S->sed_major[0];
    const float MU_MAJOR_WAVE = (TM == 0) ? MU_WAVE : (float)S->sed_major[1];
    const float COHERENT = fminf(fmaxf((float)S->muscal[7], 0.0f), 1.0f);
    const int COND = (P->event_model == 4 || P->event_model == 5);
    o_cell C = {P->n_water, P->n_acrylic, P->n_air, P->bottom_external_n, RIN, P->rout, ZMIN,
                ZMIN - P->bottom_disc_thickness, ZMEAN, ZTOP, FSM, DH, CORE};
    o_field F = {TM, FSM, S->n, S->n_radial, S->grid_nr, S->grid_nz, S->sed_A, S->sed_B, S->sed_norm,
                 S->sed_radial_log, S->sed_grid, S->grid_zmax, RIN, ZMIN, CORE};
    o_bcount bc;
    memset(&bc, 0, sizeof bc);
    float x, y, z, vx = 0.0f, vy = 1.0f, vz = 0.0f;
    int st = 0;
    /* collimated disc beam (new in this library, no reference lines to follow): a uniform disc of radius
     * disc_radius centred on the 180-degree axis at height disc_height, launched along +y from the
     * sensor-ring radius; the same two draws and arithmetic as the device's source_segment */
    if (P->source_kind == CLR_SOURCE_COLLIMATED_DISC) {
        float u1 = o_uniform(&stSRC), u2 = o_uniform(&stSRC);
        float rr = P->disc_radius * sqrtf(u1);
        float ph = 2.0f * O_PI_F * u2;
        x = rr * cosf(ph);
        z = P->disc_height + rr * sinf(ph);
        y = -P->ring_in;
    } else
    /* source (:4650-4697) */
    {
        float u1 = fmaxf(o_uniform(&stSRC), 1e-12f), u2 = o_uniform(&stSRC);
        float mag = sqrtf(-2.0f * logf(u1));
        x = P->beam_sigma * mag * cosf(2.0f * O_PI_F * u2);
        z = P->beam_sigma * mag * sinf(2.0f * O_PI_F * u2);
        y = -P->source_r;
        float polar, az;
        if (P->source_angular_model == 0) {
            polar = o_beta(&stSRC, P->alpha1, P->alpha2) * (O_PI_F / 2.0f);
            az = 2.0f * O_PI_F * o_uniform(&stSRC);
            float sp = sinf(polar);
            vx = sp * cosf(az); vy = cosf(polar); vz = sp * sinf(az);
        } else if (P->source_angular_model == 1) {
            polar = o_beta_radiance_polar(&stSRC, P->alpha1, P->alpha2);
            az = 2.0f * O_PI_F * o_uniform(&stSRC);
            float sp = sinf(polar);
            vx = sp * cosf(az); vy = cosf(polar); vz = sp * sinf(az);
        } else {
            float h = o_beta(&stSRC, P->alpha1, P->alpha2) * (O_PI_F / 2.0f);
            if (o_uniform(&stSRC) < 0.5f) h = -h;
            vx = sinf(h); vy = cosf(h); vz = 0.0f;
        }
        o_normalize(&vx, &vy, &vz);
        if (vy <= 1e-12f) { st = 3; goto done; }
        if (P->source_bore_model == 0) {
            if (x * x + z * z > P->counterbore_r * P->counterbore_r) { st = 3; goto done; }
            float t = (-P->throat_out - y) / vy;
            if (t < -O_EPS_F) { st = 3; goto done; }
            if (t < 0.0f) t = 0.0f;
            float xt = x + t * vx, zt = z + t * vz;
            if (xt * xt + zt * zt > P->throat_r * P->throat_r) { st = 3; goto done; }
            t = (-P->ring_in - y) / vy;
            if (t <= 0.0f) { st = 3; goto done; }
            x += t * vx; y += t * vy; z += t * vz;
            if (x * x + z * z > P->throat_r * P->throat_r) { st = 3; goto done; }
        } else {
            if (!o_source_collimator(&stSRC, P->source_bore_model, P->n_air, P->bore_n, P->max_bore_bounces,
                                     P->ring_in, P->throat_out, P->source_r, P->throat_r, P->counterbore_r, &x, &y, &z,
                                     &vx, &vy, &vz, &r.sbi, &r.sbr)) { st = 3; goto done; }
        }
    }
    /* air gap -> outer acrylic wall (:4700-4732) */
    {
        double tdw = o_cyl_hit_finite(x, y, z, vx, vy, vz, P->rout, ZMIN - P->bottom_disc_thickness, ZTOP);
        float t = (tdw < 0.5 * (double)O_INF_F) ? (float)tdw : O_INF_F;
        if (t >= O_INF_F * 0.5f) { st = 3; goto done; }
        x += t * vx; y += t * vy; z += t * vz;
        float nx, ny;
        o_radial_normal(x, y, &nx, &ny);
        float ci = fminf(fmaxf(-o_dot(vx, vy, vz, nx, ny, 0.0f), 0.0f), 1.0f);
        int tir = 0;
        float R = o_fresnel(ci, P->n_air, P->n_acrylic, &tir);
        float a, b, c;
        if (tir || o_uniform(&state) < R || !o_refract(vx, vy, vz, nx, ny, 0.0f, P->n_air, P->n_acrylic, &a, &b, &c)) {
            o_reflect(vx, vy, vz, nx, ny, 0.0f, &a, &b, &c);
            vx = a; vy = b; vz = c; bc.cor++; if (tir) bc.ctir++;
            x += O_EPS_F * nx; y += O_EPS_F * ny;
            st = 1; goto air_exit;
        }
        vx = a; vy = b; vz = c; x -= O_EPS_F * nx; y -= O_EPS_F * ny;
        int sub = 0, nb = 0;
        int where = o_acrylic_solid(&state, &C, C.n_air, C.n_bottom_ext, ZMIN, C.Zlow, &x, &y, &z, &vx, &vy, &vz, &r.ap,
                                    &bc, &sub, &nb);
        if (where == 2) { st = 1; goto air_exit; }
        if (where == 3) { st = 7; goto done; }
        if (where == 5) { st = 8; goto done; }
        if (where == 4) {
            int hs = 0, hb = 0;
            int hw = o_headspace(&state, &C, &x, &y, &z, &vx, &vy, &vz, &r.ap, &bc, &hs, &hb);
            if (hw == 1) r.entered = 1;
            else if (hw == 2) { st = 1; goto air_exit; }
            else if (hw == 3) { st = 7; goto done; }
            else if (hw == 4) { st = 6; goto done; }
            else if (hw == 5) { st = 8; goto done; }
            else { r.pf = OP_HEADSPACE_NO_BOUNDARY; r.pfs = hs; st = 4; goto done; }
        } else if (where != 1) {
            r.pf = (sub == OS_ACRYLIC_BOUNCE_LIMIT) ? OP_ACRYLIC_BOUNCE_LIMIT : OP_ACRYLIC_NO_INTERSECTION;
            r.pfs = sub; st = 4; goto done;
        }
        r.entered = 1;
    }
    /* water free-flight loop (:4734-5066) */
    for (int step = 0; step < (int)P->max_iterations; ++step) {
        r.steps++;
        if (!isfinite(x) || !isfinite(y) || !isfinite(z)) { r.pf = OP_NONFINITE_POSITION; r.pfs = OS_NONFINITE_POSITION; st = 4; break; }
        if (!isfinite(vx) || !isfinite(vy) || !isfinite(vz)) { r.pf = OP_NONFINITE_DIRECTION; r.pfs = OS_NONFINITE_DIRECTION; st = 4; break; }
        float zsurf_here = o_surface_z(x, y, ZMEAN, RIN, FSM, DH, CORE);
        if (z <= ZMIN || z >= zsurf_here) { st = 2; break; }
        double rr2w = (double)x * (double)x + (double)y * (double)y, ri2w = (double)RIN * (double)RIN;
        double water_tol = 8.0 * 1.1920928955078125e-7 * ri2w;
        if (rr2w > ri2w + water_tol) { r.pf = OP_INVALID_MEDIUM; r.pfs = OS_WATER_OUTSIDE; st = 4; break; }
        double tsided = o_bore_wall_hit(x, y, z, vx, vy, vz, RIN, ZMIN, ZTOP);
        if (tsided < 0.0) { r.pf = OP_INVALID_MEDIUM; r.pfs = OS_WATER_OUTSIDE; st = 4; break; }
        float tside = (tsided < 0.5 * (double)O_INF_F) ? (float)tsided : O_INF_F;
        float ttop = o_surface_hit(x, y, z, vx, vy, vz, ZMEAN, RIN, FSM, DH, CORE), tbottom = O_INF_F;
        if (vz < -1e-14f) tbottom = (ZMIN - z) / vz;
        if (!(ttop > 0.0f)) ttop = O_INF_F;
        if (!(tbottom > 0.0f)) tbottom = O_INF_F;
        int axial_top = (ttop <= tbottom && ttop < tside);
        int axial_bottom = (tbottom < ttop && tbottom < tside);
        int axial = axial_top || axial_bottom;
        float tbound = axial_top ? ttop : (axial_bottom ? tbottom : tside);
        if (tbound >= O_INF_F * 0.5f) { r.pf = OP_WATER_NO_BOUNDARY; r.pfs = OS_WATER_NO_BOUNDARY; st = 4; break; }
        float freep = O_INF_F;
        float MU_TOTAL = MU_GEOM + MU_WAVE;
        float MU_TRACK = (TM == 0) ? MU_TOTAL : (MU_MAJOR_GEOM + MU_MAJOR_WAVE);
        if (tbound > 0.0f && MU_TRACK > 0.0f) { float u = fmaxf(o_uniform(&state), 1e-12f); freep = -logf(u) / MU_TRACK; }
        int do_particle = freep < tbound;
        float travel = do_particle ? freep : tbound;
        x += travel * vx; y += travel * vy; z += travel * vz;
        r.wp += travel;
        double endpoint_r2 = (double)x * x + (double)y * y;
        if (do_particle && (endpoint_r2 > ri2w + water_tol || z < ZMIN - O_EPS_F ||
                            z > o_surface_z(x, y, ZMEAN, RIN, FSM, DH, CORE) + O_EPS_F)) {
            r.pf = OP_INVALID_MEDIUM; r.pfs = OS_WATER_OUTSIDE; st = 4; break;
        }
        if (do_particle) {
            float LOCAL_GEOM = MU_GEOM, LOCAL_WAVE = MU_WAVE, LOCAL_TOTAL = MU_TOTAL;
            if (TM != 0) {
                double lg = 0.0, lw = 0.0;
                for (int i = 0; i < S->n; ++i) {
                    double sc = o_local_scale(&F, i, x, y, z);
                    lg += S->trace_geom[i] * sc;
                    lw += S->trace_wave[i] * sc;
                }
                LOCAL_GEOM = (float)lg; LOCAL_WAVE = (float)lw; LOCAL_TOTAL = LOCAL_GEOM + LOCAL_WAVE;
                if (!(LOCAL_TOTAL > 0.0f)) { r.nulls++; continue; }
                float slack = 64.0f * 1.1920928955078125e-7f * fmaxf(fabsf(MU_TRACK), 1.0f);
                if (LOCAL_TOTAL > MU_TRACK + slack) { r.pf = OP_MAJORANT_VIOLATION; r.pfs = OS_MAJORANT; st = 4; break; }
                float pacc = LOCAL_TOTAL / fmaxf(MU_TRACK, 1e-30f);
                if (pacc > 1.0f) pacc = 1.0f;
                if (o_uniform(&state) >= pacc) { r.nulls++; continue; }
            }
            r.ic++;
            const float vinx = vx, viny = vy, vinz = vz;
            const int per0 = r.pc.entry_reflections, pir0 = r.pc.internal_reflections;
            int event_pidx = -1, event_type = 0;
            float ipath = 0.0f;
            int use_wave = (LOCAL_WAVE > 0.0f && o_uniform(&state) * LOCAL_TOTAL >= LOCAL_GEOM);
            int sel = -1;
            if (COND) {
                const double* bin_cdf = use_wave ? S->wcdf : S->gcdf;
                const double* bin_rate = use_wave ? S->trace_wave : S->trace_geom;
                sel = (TM == 0) ? o_sample_cdf(&state, bin_cdf, S->n)
                                : o_sample_local_bin(&state, &F, bin_rate, x, y, z, (double)(use_wave ? LOCAL_WAVE : LOCAL_GEOM));
            }
            if (COND && S->kidx[sel] > 0.0) {
                if ((float)S->kidx[sel] == 0.0f) { r.pf = OP_OTHER; r.pfs = 9003; st = 4; cstats[8]++; break; }
                o_hist h = o_conditional(&stOPT, sel, S->qsca[sel], S->qext[sel], P->n_water, (float)S->nidx[sel],
                                         (float)S->kidx[sel], P->wavelength, P->rough_alpha, (float)S->radius[sel],
                                         P->spheroid_aspect, P->orientation_model, P->orientation_kappa,
                                         P->max_particle_bounces, COHERENT, S->phase_cdf, S->theta, S->nt, x, y, z, vx, vy,
                                         vz, RIN, ZMIN, ZMEAN, FSM, DH, CORE, P->conditional_retries, cstats);
                event_pidx = sel;
                if (h.status != 1 && h.status != 2) { r.pf = h.failure ? h.failure : OP_OTHER; r.pfs = h.subcode; st = 4; break; }
                x = h.x; y = h.y; z = h.z; vx = h.vx; vy = h.vy; vz = h.vz;
                r.pc.reflections += h.pc.reflections; r.pc.entry_reflections += h.pc.entry_reflections;
                r.pc.internal_reflections += h.pc.internal_reflections; r.pc.absorptions += h.pc.absorptions;
                if (h.channel == 0) r.gic++;
                else { r.wic++; if (h.channel == 1) r.wcoh++; else r.wmorph++; }
                event_type = h.event_type;
                ipath = h.path;
                if (h.status == 2) {
                    o_prov_mark(&r, event_type, sel);
                    r.ipath_total += h.path;
                    r.iopl_total += h.path * (float)S->nidx[sel];
                    st = 5;
                    break;
                }
            } else if (use_wave) {
                if (COND) cstats[0]++;
                r.wic++;
                int pidx = sel >= 0 ? sel
                                    : (TM == 0) ? o_sample_cdf(&state, S->wcdf, S->n)
                                                : o_sample_local_bin(&state, &F, S->trace_wave, x, y, z, (double)LOCAL_WAVE);
                event_pidx = pidx;
                int coherent = (COHERENT >= 1.0f) || (o_uniform(&stOPT) < COHERENT);
                if (coherent) {
                    r.wcoh++;
                    o_mie_direction(&stOPT, S->phase_cdf, S->theta, S->nt, pidx, &vx, &vy, &vz);
                    if (COND) { cstats[4]++; cstats[7]++; }
                    event_type = 4;
                } else {
                    r.wmorph++;
                    float fr = sqrtf(x * x + y * y);
                    float ffx = 1.0f, ffy = 0.0f, ffz = 0.0f;
                    if (fr > 1e-12f) { ffx = -y / fr; ffy = x / fr; }
                    int ppc = 0, pps = 0, pmb = 0, pmo = 0;
                    int ps = o_spheroid_event(&stOPT, P->n_water, (float)S->nidx[pidx], (float)S->kidx[pidx], P->wavelength,
                                              P->rough_alpha, (float)S->radius[pidx], P->spheroid_aspect,
                                              P->orientation_model, P->orientation_kappa, ffx, ffy, ffz,
                                              P->max_particle_bounces, &vx, &vy, &vz, &ipath, &r.pc, &ppc, &pps, &pmb, &pmo);
                    if (ps == 2) { st = 5; break; }
                    if (ps != 1) { if (COND) cstats[8]++; r.pf = ppc ? ppc : OP_OTHER; r.pfs = pps; st = 4; break; }
                    if (COND) { cstats[5]++; cstats[7]++; }
                    event_type = (r.pc.entry_reflections > per0) ? 5 : ((r.pc.internal_reflections > pir0) ? 7 : 6);
                }
            } else {
                if (COND) cstats[0]++;
                r.gic++;
                int pidx = sel >= 0 ? sel
                                    : (TM == 0) ? o_sample_cdf(&state, S->gcdf, S->n)
                                                : o_sample_local_bin(&state, &F, S->trace_geom, x, y, z, (double)LOCAL_GEOM);
                event_pidx = pidx;
                float prad = (float)S->radius[pidx];
                float srho, sphi, sgx, sgy, sgz;
                o_sphere_geometry(&stOPT, prad, x, y, z, vx, vy, vz, &srho, &sphi, &sgx, &sgy, &sgz);
                double dscx = (double)x - (double)prad * (double)sgx;
                double dscy = (double)y - (double)prad * (double)sgy;
                double dscz = (double)z - (double)prad * (double)sgz;
                int accessible = o_sphere_accessible(dscx, dscy, dscz, (double)prad, RIN, ZMIN, ZMEAN, FSM, DH, CORE);
                if (!accessible && COND) {
                    cstats[2]++;
                    o_hist h = o_conditional(&stOPT, pidx, S->qsca[pidx], S->qext[pidx], P->n_water, (float)S->nidx[pidx],
                                             (float)S->kidx[pidx], P->wavelength, P->rough_alpha, prad, P->spheroid_aspect,
                                             P->orientation_model, P->orientation_kappa, P->max_particle_bounces,
                                             COHERENT, S->phase_cdf, S->theta, S->nt, x, y, z, vx, vy, vz, RIN, ZMIN,
                                             ZMEAN, FSM, DH, CORE, P->conditional_retries - 1, cstats);
                    if (h.status != 1) { r.pf = h.failure ? h.failure : OP_OTHER; r.pfs = h.subcode; st = 4; break; }
                    x = h.x; y = h.y; z = h.z; vx = h.vx; vy = h.vy; vz = h.vz;
                    r.pc.reflections += h.pc.reflections; r.pc.entry_reflections += h.pc.entry_reflections;
                    r.pc.internal_reflections += h.pc.internal_reflections; r.pc.absorptions += h.pc.absorptions;
                    r.gic--;
                    if (h.channel == 0) r.gic++;
                    else { r.wic++; if (h.channel == 1) r.wcoh++; else r.wmorph++; }
                    event_type = h.event_type;
                    ipath = h.path;
                } else {
                    if (!accessible) { r.ic--; r.gic--; r.nulls++; continue; }
                    int ppc = 0, pps = 0, pmb = 0, pmo = 0;
                    int ps = o_sphere_sampled(&stOPT, P->n_water, (float)S->nidx[pidx], (float)S->kidx[pidx], P->wavelength,
                                              P->rough_alpha, prad, P->max_particle_bounces, sgx, sgy, sgz, dscx, dscy,
                                              dscz, &x, &y, &z, &vx, &vy, &vz, &ipath, &r.pc, &ppc, &pps, &pmb, &pmo);
                    if (ps == 2) { st = 5; break; }
                    if (ps != 1) { if (COND) cstats[8]++; r.pf = ppc ? ppc : OP_OTHER; r.pfs = pps; st = 4; break; }
                    if (COND) { cstats[3]++; cstats[7]++; }
                    event_type = (r.pc.entry_reflections > per0) ? 1 : ((r.pc.internal_reflections > pir0) ? 3 : 2);
                }
            }
            if (event_pidx >= 0 && S->moment_mode[event_pidx])
                o_moment(vinx, viny, vinz, &vx, &vy, &vz, (float)S->moment_a[event_pidx], (float)S->moment_b[event_pidx]);
            /* provenance of the survived event (:4949-4979) */
            {
                const float dcos = fminf(fmaxf(o_dot(vinx, viny, vinz, vx, vy, vz), -1.0f), 1.0f);
                const float defl = acosf(dcos) * (180.0f / O_PI_F);
                r.ipath_total += ipath;
                if (event_pidx >= 0) r.iopl_total += ipath * (float)S->nidx[event_pidx];
                o_prov_mark(&r, event_type, event_pidx);
                r.last_defl = defl;
                r.wp_last = r.wp;
                if (r.ic == 1) { r.first_defl = defl; r.first_back = dcos < 0.0f; r.first_hemi = vy < 0.0f; }
            }
            continue;
        }
        if (axial) {
            float a, b, c;
            int tir = 0;
            if (axial_top) {
                float snx = 0.0f, sny = 0.0f, snz = -1.0f;
                o_surface_normal(x, y, RIN, FSM, DH, CORE, &snx, &sny, &snz);
                float ci = fminf(fmaxf(-o_dot(vx, vy, vz, snx, sny, snz), 0.0f), 1.0f);
                float R = o_fresnel(ci, P->n_water, P->n_air, &tir);
                if (tir || o_uniform(&state) < R || !o_refract(vx, vy, vz, snx, sny, snz, P->n_water, P->n_air, &a, &b, &c)) {
                    o_reflect(vx, vy, vz, snx, sny, snz, &a, &b, &c);
                    vx = a; vy = b; vz = c; bc.tr++; if (tir) bc.ttir++;
                    if (!o_surface_offset(&x, &y, &z, snx, sny, snz, RIN, ZMIN, ZMEAN, FSM, DH, CORE)) {
                        r.pf = OP_INVALID_MEDIUM; r.pfs = OS_WATER_OUTSIDE; st = 4; break;
                    }
                    continue;
                }
                vx = a; vy = b; vz = c;
                x -= O_EPS_F * snx; y -= O_EPS_F * sny; z -= O_EPS_F * snz;
                int hs = 0, hb = 0;
                int hw = o_headspace(&state, &C, &x, &y, &z, &vx, &vy, &vz, &r.ap, &bc, &hs, &hb);
                if (hw == 1) { if (r.ic > 0) r.acr_returns++; continue; }
                if (hw == 2) { st = 1; goto air_exit; }
                if (hw == 3) { st = 7; goto done; }
                if (hw == 4) { st = 6; goto done; }
                r.pf = OP_HEADSPACE_NO_BOUNDARY; r.pfs = hs; st = 4; goto done;
            } else {
                int bs = 0, bb = 0;
                int where = o_bottom_disc(&state, &C, &x, &y, &z, &vx, &vy, &vz, &r.ap, &bc, &bs, &bb);
                if (where == 1) { if (r.ic > 0) r.acr_returns++; continue; }
                if (where == 2) { st = 1; goto air_exit; }
                if (where == 3) { st = 7; break; }
                if (where == 5) { st = 8; break; }
                if (where == 4) {
                    int hs = 0, hb = 0;
                    int hw = o_headspace(&state, &C, &x, &y, &z, &vx, &vy, &vz, &r.ap, &bc, &hs, &hb);
                    if (hw == 1) { if (r.ic > 0) r.acr_returns++; continue; }
                    if (hw == 2) { st = 1; goto air_exit; }
                    if (hw == 3) { st = 7; goto done; }
                    if (hw == 4) { st = 6; goto done; }
                    r.pf = OP_HEADSPACE_NO_BOUNDARY; r.pfs = hs; st = 4; goto done;
                }
                r.pf = (bs == OS_ACRYLIC_BOUNCE_LIMIT) ? OP_ACRYLIC_BOUNCE_LIMIT : OP_BOTTOM_GEOMETRY;
                r.pfs = bs; st = 4; break;
            }
        }
        /* water -> acrylic at the cylinder wall (:5038-5065) */
        {
            float nx, ny;
            o_radial_normal(x, y, &nx, &ny);
            float ci = fminf(fmaxf(o_dot(vx, vy, vz, nx, ny, 0.0f), 0.0f), 1.0f);
            int tir = 0;
            float R = o_fresnel(ci, P->n_water, P->n_acrylic, &tir);
            float a, b, c;
            if (tir || o_uniform(&state) < R || !o_refract(vx, vy, vz, -nx, -ny, 0.0f, P->n_water, P->n_acrylic, &a, &b, &c)) {
                o_reflect(vx, vy, vz, nx, ny, 0.0f, &a, &b, &c);
                vx = a; vy = b; vz = c; bc.cir++; if (tir) bc.ctir++;
                x -= O_EPS_F * nx; y -= O_EPS_F * ny;
                continue;
            }
            vx = a; vy = b; vz = c; x += O_EPS_F * nx; y += O_EPS_F * ny;
            int sub = 0, nb = 0;
            int where = o_acrylic_solid(&state, &C, C.n_air, C.n_bottom_ext, ZMIN, C.Zlow, &x, &y, &z, &vx, &vy, &vz,
                                        &r.ap, &bc, &sub, &nb);
            if (where == 1) { if (r.ic > 0) r.acr_returns++; continue; }
            if (where == 2) { st = 1; goto air_exit; }
            if (where == 3) { st = 7; break; }
            if (where == 5) { st = 8; break; }
            if (where == 4) {
                int hs = 0, hb = 0;
                int hw = o_headspace(&state, &C, &x, &y, &z, &vx, &vy, &vz, &r.ap, &bc, &hs, &hb);
                if (hw == 1) { if (r.ic > 0) r.acr_returns++; continue; }
                if (hw == 2) { st = 1; goto air_exit; }
                if (hw == 3) { st = 7; goto done; }
                if (hw == 4) { st = 6; goto done; }
                if (hw == 5) { st = 8; goto done; }
                r.pf = OP_HEADSPACE_NO_BOUNDARY; r.pfs = hs; st = 4; goto done;
            }
            r.pf = (sub == OS_ACRYLIC_BOUNCE_LIMIT) ? OP_ACRYLIC_BOUNCE_LIMIT : OP_ACRYLIC_NO_INTERSECTION;
            r.pfs = sub; st = 4; break;
        }
    }
    if (st == 0) { r.pf = OP_ITERATION_LIMIT; r.pfs = OS_ITERATION_LIMIT; st = 4; }
    goto done;
air_exit:
    r.ax = x; r.ay = y; r.az = z; r.avx = vx; r.avy = vy; r.avz = vz;
done:
    r.st = st;
    r.cir = bc.cir; r.cor = bc.cor; r.ctir = bc.ctir; r.tr = bc.tr; r.ttir = bc.ttir;
    r.bir = bc.bir; r.bor = bc.bor; r.btir = bc.btir;
    *out = r;
}

/* ---------------- detectors (:4237-4376) ---------------- */
static int o_hardware_detector(float x, float y, float z, float vx, float vy, float vz, int mirror, float ring_in,
                               float throat_out, float ring_out, float throat_r, float counterbore_r) {
    if (mirror) { x = -x; vx = -vx; }
    float best_t = O_INF_F;
    int best = -1;
    float rth2 = throat_r * throat_r, rcb2 = counterbore_r * counterbore_r;
    for (int j = 0; j < 18; ++j) {
        float th = o_det_theta(j), ux = sinf(th), uy = cosf(th);
        float den = vx * ux + vy * uy;
        if (den <= 1e-10f) continue;
        float pdot = x * ux + y * uy;
        float t0 = (ring_in - pdot) / den, t1 = (throat_out - pdot) / den, t2 = (ring_out - pdot) / den;
        if (!(t0 > 0.0f && t1 > t0 && t2 > t1)) continue;
        float q0x = x + t0 * vx - ring_in * ux, q0y = y + t0 * vy - ring_in * uy, q0z = z + t0 * vz;
        float q1x = x + t1 * vx - throat_out * ux, q1y = y + t1 * vy - throat_out * uy, q1z = z + t1 * vz;
        float q2x = x + t2 * vx - ring_out * ux, q2y = y + t2 * vy - ring_out * uy, q2z = z + t2 * vz;
        if (q0x * q0x + q0y * q0y + q0z * q0z <= rth2 && q1x * q1x + q1y * q1y + q1z * q1z <= rth2 &&
            q2x * q2x + q2y * q2y + q2z * q2z <= rcb2) {
            if (t0 < best_t) { best_t = t0; best = j; }
        }
    }
    return best;
}
static float o_sfh213(float phi_deg) {
    const float HALF_DEG = 10.0f, PW = 3.169925001442312f;
    float a = fabsf(phi_deg);
    if (a >= 90.0f) return 0.0f;
    float u = a / HALF_DEG;
    return 1.0f / (1.0f + powf(u, PW));
}
static float o_incidence_deg(float vx, float vy, float vz, int id, int mirror) {
    (void)vz;
    if (id < 0 || id >= 18) return -1.0f;
    if (mirror) vx = -vx;
    float th = o_det_theta(id);
    float ux = sinf(th), uy = cosf(th);
    float c = vx * ux + vy * uy;
    c = fminf(fmaxf(c, -1.0f), 1.0f);
    return acosf(c) * (180.0f / O_PI_F);
}
static int o_throat_opening(float x, float y, float z, float vx, float vy, float vz, float ring_in, float throat_r) {
    float best_t = O_INF_F;
    int best = -1;
    float r2 = throat_r * throat_r;
    for (int j = 0; j < 19; ++j) {
        float th = o_det_theta(j), ux = sinf(th), uy = cosf(th);
        float den = vx * ux + vy * uy;
        if (den <= 1.0e-10f) continue;
        float pdot = x * ux + y * uy;
        float t = (ring_in - pdot) / den;
        if (t <= 0.0f) continue;
        float qx = x + t * vx - ring_in * ux, qy = y + t * vy - ring_in * uy, qz = z + t * vz;
        if (qx * qx + qy * qy + qz * qz <= r2 && t < best_t) { best_t = t; best = j; }
    }
    return best;
}
static float o_cylinder_hit(float x, float y, float vx, float vy, float R) {
    float a = vx * vx + vy * vy;
    if (a < 1e-18f) return O_INF_F;
    float b = x * vx + y * vy;
    float c = x * x + y * y - R * R;
    float d = b * b - a * c;
    if (d < 0.0f) return O_INF_F;
    float sd = sqrtf(fmaxf(d, 0.0f));
    float t1 = (-b - sd) / a, t2 = (-b + sd) / a;
    float t = O_INF_F;
    if (t1 > O_EPS_F) t = t1;
    if (t2 > O_EPS_F && t2 < t) t = t2;
    return t;
}
static int o_ring_face_path(uint32_t* s, float x, float y, float z, float vx, float vy, float vz, int mirror,
                            const clr_scene_params* P, int* bore_bounces, int* face_reflections) {
    if (mirror) { x = -x; vx = -vx; }
    *bore_bounces = 0;
    *face_reflections = 0;
    if (P->ring_face_model == 0) return -1;
    if (o_throat_opening(x, y, z, vx, vy, vz, P->ring_in, P->throat_r) >= 0) return -1;
    for (int b = 0; b < P->max_ring_face_bounces; ++b) {
        float tr = o_cylinder_hit(x, y, vx, vy, P->ring_in);
        if (tr >= O_INF_F * 0.5f) return -1;
        x += tr * vx; y += tr * vy; z += tr * vz;
        float nx, ny;
        o_radial_normal(x, y, &nx, &ny);
        float ci = fminf(fmaxf(vx * nx + vy * ny, 0.0f), 1.0f);
        int tir = 0;
        float R = o_fresnel(ci, P->n_air, P->ring_face_n, &tir);
        if (o_uniform(s) >= R) return -1;
        float a, c, d;
        o_reflect(vx, vy, vz, -nx, -ny, 0.0f, &a, &c, &d);
        vx = a; vy = c; vz = d;
        (*face_reflections)++;
        x -= O_EPS_F * nx; y -= O_EPS_F * ny;
        float ta = o_cylinder_hit(x, y, vx, vy, P->rout);
        if (ta >= O_INF_F * 0.5f) return -1;
        x += ta * vx; y += ta * vy; z += ta * vz;
        o_radial_normal(x, y, &nx, &ny);
        ci = fminf(fmaxf(-o_dot(vx, vy, vz, nx, ny, 0.0f), 0.0f), 1.0f);
        R = o_fresnel(ci, P->n_air, P->n_acrylic, &tir);
        if (o_uniform(s) >= R) return -1;
        o_reflect(vx, vy, vz, nx, ny, 0.0f, &a, &c, &d);
        vx = a; vy = c; vz = d;
        x += O_EPS_F * nx; y += O_EPS_F * ny;
        int db = 0, det;
        if (P->detector_bore_model == 0)
            det = o_hardware_detector(x, y, z, vx, vy, vz, 0, P->ring_in, P->throat_out, P->ring_out, P->throat_r, P->counterbore_r);
        else
            det = o_detector_collimator_path(s, x, y, z, vx, vy, vz, 0, P->ring_in, P->throat_out, P->ring_out, P->throat_r,
                                             P->counterbore_r, P->detector_bore_model, P->n_air, P->bore_n,
                                             P->max_bore_bounces, &db);
        if (det >= 0) { *bore_bounces = db; return det; }
        if (o_throat_opening(x, y, z, vx, vy, vz, P->ring_in, P->throat_r) >= 0) return -1;
    }
    return -1;
}

/* score one ray (:4390-4436); accumulates into T */
static void o_score(const clr_scene_params* P, uint32_t detector_seed, uint32_t gid, const o_ray* r, clr_tallies* T,
                    clr_ray_record* rec) {
    int ni = -1, mi = -1, nb = 0, mb = 0, nfb = 0, mfb = 0;
    if (rec) { rec->native_id = -1; rec->mirror_id = -1; rec->native_bounces = 0; rec->mirror_bounces = 0; }
    if (r->st != 1) return;
    float x = r->ax, y = r->ay, z = r->az, vx = r->avx, vy = r->avy, vz = r->avz;
    if (!(isfinite(x) && isfinite(y) && isfinite(z) && isfinite(vx) && isfinite(vy) && isfinite(vz))) return;
    uint32_t sN = detector_seed + gid * 2246822519u + 3266489917u;
    uint32_t sM = detector_seed + gid * 3266489917u + 668265263u;
    if (P->detector_bore_model == 0) {
        ni = o_hardware_detector(x, y, z, vx, vy, vz, 0, P->ring_in, P->throat_out, P->ring_out, P->throat_r, P->counterbore_r);
        mi = o_hardware_detector(x, y, z, vx, vy, vz, 1, P->ring_in, P->throat_out, P->ring_out, P->throat_r, P->counterbore_r);
    } else {
        ni = o_detector_collimator_path(&sN, x, y, z, vx, vy, vz, 0, P->ring_in, P->throat_out, P->ring_out, P->throat_r,
                                        P->counterbore_r, P->detector_bore_model, P->n_air, P->bore_n, P->max_bore_bounces, &nb);
        mi = o_detector_collimator_path(&sM, x, y, z, vx, vy, vz, 1, P->ring_in, P->throat_out, P->ring_out, P->throat_r,
                                        P->counterbore_r, P->detector_bore_model, P->n_air, P->bore_n, P->max_bore_bounces, &mb);
    }
    if (ni < 0 && P->ring_face_model != 0) ni = o_ring_face_path(&sN, x, y, z, vx, vy, vz, 0, P, &nb, &nfb);
    if (mi < 0 && P->ring_face_model != 0) mi = o_ring_face_path(&sM, x, y, z, vx, vy, vz, 1, P, &mb, &mfb);
    if (rec) { rec->native_id = ni; rec->mirror_id = mi; rec->native_bounces = nb; rec->mirror_bounces = mb; }
    if (ni >= 0) {
        T->hw_native[ni]++;
        if (nb > 0 || nfb > 0) T->hw_native_stray[ni]++; else T->hw_native_direct[ni]++;
        if (nfb > 0) T->hw_native_face[ni]++;
        T->weight_native[ni] += 1.0; T->weight_sq_native[ni] += 1.0;
        float phi = o_incidence_deg(vx, vy, vz, ni, 0);
        if (phi >= 0.0f && isfinite(phi)) {
            float resp = (P->photodiode_model == 0) ? 1.0f : o_sfh213(phi);
            T->photodiode_native[ni] += resp;
            T->incidence_native_sum[ni] += phi;
        }
    }
    if (mi >= 0) {
        T->hw_mirror[mi]++;
        if (mb > 0 || mfb > 0) T->hw_mirror_stray[mi]++; else T->hw_mirror_direct[mi]++;
        if (mfb > 0) T->hw_mirror_face[mi]++;
        T->weight_mirror[mi] += 1.0; T->weight_sq_mirror[mi] += 1.0;
        float phi = o_incidence_deg(vx, vy, vz, mi, 1);
        if (phi >= 0.0f && isfinite(phi)) {
            float resp = (P->photodiode_model == 0) ? 1.0f : o_sfh213(phi);
            T->photodiode_mirror[mi] += resp;
            T->incidence_mirror_sum[mi] += phi;
        }
    }
    for (int mirror = 0; mirror < 2; ++mirror) {
        float xx = mirror ? -x : x;
        float ang = atan2f(xx, y) * (180.0f / O_PI_F);
        if (ang < 0.0f) ang += 360.0f;
        if (ang < 0.0f || ang > 180.0f) continue;
        for (int j = 0; j < 18; ++j) {
            float deg = 10.0f * j;
            if (r->ic <= 0 && deg >= 90.0f) continue;
            if (fabsf(ang - deg) <= P->legacy_accept_deg) {
                if (mirror) T->legacy_mirror[j]++; else T->legacy_native[j]++;
            }
        }
    }
}

static void tally_merge(clr_tallies* dst, const clr_tallies* src) {
    int64_t* d = (int64_t*)dst;
    const int64_t* s = (const int64_t*)src;
    /* integer blocks */
    for (int j = 0; j < 18; ++j) {
        dst->hw_native[j] += src->hw_native[j]; dst->hw_mirror[j] += src->hw_mirror[j];
        dst->hw_native_direct[j] += src->hw_native_direct[j]; dst->hw_mirror_direct[j] += src->hw_mirror_direct[j];
        dst->hw_native_stray[j] += src->hw_native_stray[j]; dst->hw_mirror_stray[j] += src->hw_mirror_stray[j];
        dst->hw_native_face[j] += src->hw_native_face[j]; dst->hw_mirror_face[j] += src->hw_mirror_face[j];
        dst->legacy_native[j] += src->legacy_native[j]; dst->legacy_mirror[j] += src->legacy_mirror[j];
        dst->photodiode_native[j] += src->photodiode_native[j]; dst->photodiode_mirror[j] += src->photodiode_mirror[j];
        dst->incidence_native_sum[j] += src->incidence_native_sum[j]; dst->incidence_mirror_sum[j] += src->incidence_mirror_sum[j];
        dst->weight_native[j] += src->weight_native[j]; dst->weight_mirror[j] += src->weight_mirror[j];
        dst->weight_sq_native[j] += src->weight_sq_native[j]; dst->weight_sq_mirror[j] += src->weight_sq_mirror[j];
    }
    for (int k = 0; k < CLR_N_STATUS; ++k) dst->status_counts[k] += src->status_counts[k];
    for (int k = 0; k < CLR_N_FAILURE_CODES; ++k) dst->failure_code_counts[k] += src->failure_code_counts[k];
    for (int k = 0; k < CLR_N_EVENT_COUNTERS; ++k) dst->event_counts[k] += src->event_counts[k];
    clr_tally_merge_extras(dst, src);
    (void)d; (void)s;
}

static int trace_impl(clo_state* S, const clr_run_params* run, clr_tallies* T, clr_ray_record* records,
                      int32_t* prov, float* defl, int n_threads);

int clo_trace(clo_state* S, const clr_run_params* run, clr_tallies* T, clr_ray_record* records, int n_threads) {
    return trace_impl(S, run, T, records, NULL, NULL, n_threads);
}

int clo_trace_provenance(clo_state* S, const clr_run_params* run, clr_tallies* T, clr_ray_record* records,
                         int32_t* prov, float* defl, int n_threads) {
    return trace_impl(S, run, T, records, prov, defl, n_threads);
}

static int trace_impl(clo_state* S, const clr_run_params* run, clr_tallies* T, clr_ray_record* records,
                      int32_t* prov, float* defl, int n_threads) {
    if (!S || !run || !T) return -1;
    if (run->rng_mode != CLR_RNG_REFERENCE_XORSHIFT || run->weight_mode != CLR_WEIGHT_ANALOG) {
        snprintf(S->err, sizeof S->err, "the oracle restates xorshift streams and analog weights only");
        return -4;
    }
    memset(T, 0, sizeof *T);
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
    unsigned long long cstats[10] = {0};
    const int64_t n = run->n_rays;
#pragma omp parallel
    {
        clr_tallies* Lp = (clr_tallies*)calloc(1, sizeof(clr_tallies));
        clr_tallies L_dummy;
        (void)L_dummy;
#define L (*Lp)
        unsigned long long cs[10] = {0};
#pragma omp for schedule(dynamic, 1024)
        for (int64_t i = 0; i < n; ++i) {
            uint32_t gid = run->ray_offset + (uint32_t)i;
            o_ray r;
            o_trace_ray(S, gid, run->seed0, run->seed1, run->seed2, cs, &r);
            clr_ray_record tmp;
            memset(&tmp, 0, sizeof tmp);
            clr_ray_record* rec = &tmp;
            o_score(&S->sp, run->detector_seed, gid, &r, &L, rec);
            if (r.st >= 0 && r.st < CLR_N_STATUS) L.status_counts[r.st]++;
            if (r.pf >= 0 && r.pf < CLR_N_FAILURE_CODES) L.failure_code_counts[r.pf]++;
            int ev[20] = {r.ic, r.gic, r.wic, r.wcoh, r.wmorph, r.pc.reflections, r.pc.entry_reflections,
                          r.pc.internal_reflections, r.pc.absorptions, r.cir, r.cor, r.ctir, r.tr, r.ttir, r.bir, r.bor,
                          r.btir, r.sbi, r.sbr, r.entered};
            for (int k = 0; k < 20; ++k) L.event_counts[k] += ev[k];
            L.event_counts[CLR_EV_WATER_STEPS] += r.steps;
            L.event_counts[CLR_EV_NULL_COLLISIONS] += r.nulls;
            rec->status = r.st;
            int32_t* ri = &rec->interaction_count;
            for (int k = 0; k < 20; ++k) ri[k] = ev[k];
            rec->failure_code = r.pf; rec->failure_subcode = r.pfs;
            rec->air_x = r.ax; rec->air_y = r.ay; rec->air_z = r.az;
            rec->air_vx = r.avx; rec->air_vy = r.avy; rec->air_vz = r.avz;
            rec->water_path = r.wp; rec->acrylic_path = r.ap;
            clr_tally_add_ray_stats(&L, rec);
            if (records) records[i] = tmp;
            if (prov) {
                const int32_t v[13] = {r.first_evt, r.last_evt, r.last_order, r.first_back, r.first_hemi, r.bins[0],
                                       r.bins[1], r.bins[2], r.bins[3], r.bins[4], r.bins[5], r.acr_returns,
                                       r.after_return};
                memcpy(prov + i * 13, v, sizeof v);
            }
            if (defl) {
                float* d = defl + i * 5;
                d[0] = r.first_defl; d[1] = r.last_defl; d[2] = r.ipath_total; d[3] = r.iopl_total;
                d[4] = (r.last_order > 0 && r.wp_last >= 0.0f) ? fmaxf(r.wp - r.wp_last, 0.0f) : -1.0f;
            }
        }
#pragma omp critical
        {
            tally_merge(T, &L);
            for (int k = 0; k < 10; ++k) cstats[k] += cs[k];
        }
#undef L
        free(Lp);
    }
    T->n_rays = n;
    for (int k = 0; k < 10; ++k) T->conditional_stats[k] = cstats[k];
    return 0;
}

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC11):
 * ten rounds of two 32x32->64 multiplies with the published multipliers and Weyl key increments. */
int clo_philox4x32_10(const uint32_t key[2], const uint32_t ctr[4], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3], k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0, n1 = (uint32_t)p1, n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1, n3 = (uint32_t)p0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
    return 0;
}
