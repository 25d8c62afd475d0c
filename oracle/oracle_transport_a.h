/* CPU oracle, part A: random streams, samplers, ray optics, collimator bores,
 * complex-index interfaces, free surfaces, sediment field lookup and polynomial
 * roots. Test infrastructure only (see claritas_oracle.c).
 *
 * This is a plain-C restatement of the reference's device functions. Where the
 * reference's floating-point operation order decides a branch, the same order
 * is kept so that, compiled without FMA contraction, the oracle reproduces the
 * host build of the reference bit for bit. Each function names the reference
 * lines it restates (file CLARITAS/CLARITAS.py).
 */
#ifndef CLARITAS_ORACLE_TRANSPORT_A_H
#define CLARITAS_ORACLE_TRANSPORT_A_H

#include <math.h>
#include <stdint.h>
#include <string.h>
#include "oracle_math.h"

#define O_INF_F 3.402823466e+38F          /* :1121, FLT_MAX used as "no hit" */
#define O_PI_F 3.14159265358979323846f
#define O_EPS_F 2.0e-7f
#define O_PI_D 3.141592653589793238462643383279502884
#define O_DBL_EPS 2.220446049250313080847263336181640625e-16
#define O_FLT_EPS 1.1920928955078125e-7

/* ---------------- random streams (:1125-1133, :1908-1912, :4486-4490) ---------------- */
static inline uint32_t o_next(uint32_t* s) {
    uint32_t x = *s;
    x ^= x << 13; x ^= x >> 17; x ^= x << 5;
    *s = x;
    return x;
}
static inline float o_uniform(uint32_t* s) { return (float)o_next(s) * 2.3283064e-10f; }
static inline double o_open_uniform(uint32_t* s) {
    uint32_t r = o_next(s);
    return ((double)r + 0.5) * 2.3283064365386962890625e-10;
}
static inline double o_uniform53(uint32_t* s) {
    uint32_t a = o_next(s), b = o_next(s);
    return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * 1.11022302462515654042e-16;
}

static inline float o_rsqrtf(float q) { return 1.0f / sqrtf(q); }

/* ---------------- samplers (:1148-1212) ---------------- */
static inline float o_normal(uint32_t* s) {
    float u1 = fmaxf(o_uniform(s), 1e-12f), u2 = o_uniform(s);
    return sqrtf(-2.0f * logf(u1)) * cosf(2.0f * O_PI_F * u2);
}
static float o_gamma(uint32_t* s, float shape) {
    if (shape <= 0.0f) return 0.0f;
    if (fabsf(shape - 1.0f) < 1e-7f) return -logf(fmaxf(o_uniform(s), 1e-12f));
    float correction = 1.0f, a = shape;
    if (a < 1.0f) {
        float u = fmaxf(o_uniform(s), 1e-12f);
        correction = powf(u, 1.0f / a);
        a += 1.0f;
    }
    float d = a - 0.3333333333333333f;
    float c = o_rsqrtf(9.0f * d);
    for (int it = 0; it < 128; ++it) {
        float x = o_normal(s);
        float v = 1.0f + c * x;
        if (v <= 0.0f) continue;
        v = v * v * v;
        float u = o_uniform(s);
        if (u < 1.0f - 0.0331f * x * x * x * x) return correction * d * v;
        if (logf(fmaxf(u, 1e-12f)) < 0.5f * x * x + d * (1.0f - v + logf(v))) return correction * d * v;
    }
    return correction * d;
}
static float o_beta(uint32_t* s, float a, float b) {
    if (a <= 0.0f || b <= 0.0f) return 0.0f;
    if (fabsf(a - 1.0f) < 1e-7f) {
        float u = fminf(fmaxf(o_uniform(s), 1e-12f), 1.0f - 1e-7f);
        return 1.0f - powf(1.0f - u, 1.0f / b);
    }
    if (fabsf(b - 1.0f) < 1e-7f) {
        float u = fminf(fmaxf(o_uniform(s), 1e-12f), 1.0f - 1e-7f);
        return powf(u, 1.0f / a);
    }
    float ga = o_gamma(s, a), gb = o_gamma(s, b);
    float t = ga + gb;
    return t > 0.0f ? ga / t : 0.0f;
}
/* Beta angular-radiance polar angle, rejection by sin(x)/x (:1201-1212) */
static float o_beta_radiance_polar(uint32_t* s, float a, float b) {
    const float c = 0.5f * O_PI_F;
    for (int it = 0; it < 128; ++it) {
        float u = o_beta(s, a + 1.0f, b);
        u = fminf(fmaxf(u, 0.0f), 1.0f);
        float x = c * u;
        float accept = (x < 1.0e-7f) ? 1.0f : sinf(x) / x;
        if (o_uniform(s) <= accept) return x;
    }
    float u = o_beta(s, a + 1.0f, b);
    return c * fminf(fmaxf(u, 0.0f), 1.0f);
}

/* ---------------- vectors and Fresnel (:1214-1260) ---------------- */
static inline float o_dot(float ax, float ay, float az, float bx, float by, float bz) {
    return ax * bx + ay * by + az * bz;
}
static inline void o_normalize(float* x, float* y, float* z) {
    float q = (*x) * (*x) + (*y) * (*y) + (*z) * (*z);
    if (q <= 0.0f) { *x = 0.0f; *y = 1.0f; *z = 0.0f; return; }
    float s = o_rsqrtf(q);
    *x *= s; *y *= s; *z *= s;
}
static inline void o_reflect(float ix, float iy, float iz, float nx, float ny, float nz, float* ox, float* oy, float* oz) {
    float d = o_dot(ix, iy, iz, nx, ny, nz);
    *ox = ix - 2.0f * d * nx; *oy = iy - 2.0f * d * ny; *oz = iz - 2.0f * d * nz;
    o_normalize(ox, oy, oz);
}
/* n points into the incident medium; returns 0 on total internal reflection */
static inline int o_refract(float ix, float iy, float iz, float nx, float ny, float nz, float n1, float n2,
                            float* ox, float* oy, float* oz) {
    float ci = -o_dot(ix, iy, iz, nx, ny, nz);
    ci = fminf(fmaxf(ci, 0.0f), 1.0f);
    float eta = n1 / n2;
    float k = 1.0f - eta * eta * (1.0f - ci * ci);
    if (k <= 0.0f) return 0;
    float ct = sqrtf(k);
    *ox = eta * ix + (eta * ci - ct) * nx;
    *oy = eta * iy + (eta * ci - ct) * ny;
    *oz = eta * iz + (eta * ci - ct) * nz;
    o_normalize(ox, oy, oz);
    return 1;
}
static inline float o_fresnel(float ci, float n1, float n2, int* tir) {
    ci = fminf(fmaxf(ci, 0.0f), 1.0f);
    float eta = n1 / n2;
    float st2 = eta * eta * fmaxf(0.0f, 1.0f - ci * ci);
    if (st2 >= 1.0f) { *tir = 1; return 1.0f; }
    *tir = 0;
    float ct = sqrtf(fmaxf(0.0f, 1.0f - st2));
    float ds = n1 * ci + n2 * ct, dp = n1 * ct + n2 * ci;
    float rs = 1.0f, rp = 1.0f;
    if (fabsf(ds) > 1e-12f) { float a = (n1 * ci - n2 * ct) / ds; rs = a * a; }
    if (fabsf(dp) > 1e-12f) { float a = (n1 * ct - n2 * ci) / dp; rp = a * a; }
    return fminf(fmaxf(0.5f * (rs + rp), 0.0f), 1.0f);
}
static inline void o_radial_normal(float x, float y, float* nx, float* ny) {
    float r = sqrtf(fmaxf(x * x + y * y, 1e-30f));
    *nx = x / r; *ny = y / r;
}

/* ---------------- collimator bores (:1263-1374) ---------------- */
static inline float o_bore_side_hit(float q, float w, float vq, float vw, float radius) {
    float A = vq * vq + vw * vw;
    if (A <= 1.0e-20f) return O_INF_F;
    float B = 2.0f * (q * vq + w * vw);
    float Cc = q * q + w * w - radius * radius;
    float D = B * B - 4.0f * A * Cc;
    if (D < 0.0f) return O_INF_F;
    float root = sqrtf(fmaxf(D, 0.0f));
    float t1 = (-B - root) / (2.0f * A), t2 = (-B + root) / (2.0f * A);
    float t = O_INF_F;
    if (t1 > O_EPS_F) t = t1;
    if (t2 > O_EPS_F && t2 < t) t = t2;
    return t;
}
static int o_bore_wall_reflect(uint32_t* s, int model, float n_air, float n_bore, float q, float w, float* vs,
                               float* vq, float* vw, int* interactions, int* reflections) {
    (*interactions)++;
    if (model == 0) return 0;
    float rr = sqrtf(fmaxf(q * q + w * w, 1.0e-30f));
    float ns = 0.0f, nq = -q / rr, nw = -w / rr;
    float ci = fminf(fmaxf(-((*vs) * ns + (*vq) * nq + (*vw) * nw), 0.0f), 1.0f);
    int tir = 0;
    float R = o_fresnel(ci, n_air, n_bore, &tir);
    if (o_uniform(s) >= R) return 0;
    float os, oq, ow;
    o_reflect(*vs, *vq, *vw, ns, nq, nw, &os, &oq, &ow);
    *vs = os; *vq = oq; *vw = ow;
    (*reflections)++;
    return 1;
}
static int o_bore_segment(uint32_t* st, int model, float n_air, float n_bore, int max_bounces, float s_end,
                          float radius, float* s, float* q, float* w, float* vs, float* vq, float* vw,
                          int* interactions, int* reflections) {
    for (int b = 0; b <= max_bounces; ++b) {
        if (*vs <= 1.0e-12f) return 0;
        float tp = (s_end - *s) / (*vs);
        if (tp < -O_EPS_F) return 0;
        if (tp < 0.0f) tp = 0.0f;
        float twall = o_bore_side_hit(*q, *w, *vq, *vw, radius);
        if (tp <= twall) {
            *q += tp * (*vq); *w += tp * (*vw); *s = s_end;
            return ((*q) * (*q) + (*w) * (*w) <= radius * radius * (1.0f + 2.0e-5f));
        }
        if (twall >= O_INF_F * 0.5f) return 0;
        *q += twall * (*vq); *w += twall * (*vw); *s += twall * (*vs);
        if (!o_bore_wall_reflect(st, model, n_air, n_bore, *q, *w, vs, vq, vw, interactions, reflections)) return 0;
        float rr = sqrtf(fmaxf((*q) * (*q) + (*w) * (*w), 1.0e-30f));
        *q -= O_EPS_F * (*q) / rr; *w -= O_EPS_F * (*w) / rr;
    }
    return 0;
}
static int o_source_collimator(uint32_t* st, int model, float n_air, float n_bore, int max_bounces, float ring_in,
                               float throat_out, float source_r, float throat_r, float counterbore_r, float* x,
                               float* y, float* z, float* vx, float* vy, float* vz, int* interactions,
                               int* reflections) {
    (void)source_r;
    if (*vy <= 1.0e-12f) return 0;
    float s = *y, q = *x, w = *z, vs = *vy, vq = *vx, vw = *vz;
    if (q * q + w * w > counterbore_r * counterbore_r) return 0;
    float shoulder = -throat_out;
    if (s < shoulder - O_EPS_F) {
        if (!o_bore_segment(st, model, n_air, n_bore, max_bounces, shoulder, counterbore_r, &s, &q, &w, &vs, &vq, &vw,
                            interactions, reflections))
            return 0;
    } else if (s > shoulder + O_EPS_F) {
        return 0;
    }
    if (q * q + w * w > throat_r * throat_r) return 0;
    if (!o_bore_segment(st, model, n_air, n_bore, max_bounces, -ring_in, throat_r, &s, &q, &w, &vs, &vq, &vw,
                        interactions, reflections))
        return 0;
    *x = q; *y = s; *z = w; *vx = vq; *vy = vs; *vz = vw;
    return 1;
}
/* detector direction tables: identical float arithmetic to (10*j)*(pi/180) then sinf/cosf */
static inline float o_det_theta(int j) { return (10.0f * (float)j) * (O_PI_F / 180.0f); }

static int o_detector_collimator_path(uint32_t* st, float x, float y, float z, float vx, float vy, float vz,
                                      int mirror, float ring_in, float throat_out, float ring_out, float throat_r,
                                      float counterbore_r, int model, float n_air, float n_bore, int max_bounces,
                                      int* bounce_count) {
    if (mirror) { x = -x; vx = -vx; }
    float best_t = O_INF_F;
    int best = -1;
    for (int j = 0; j < 18; ++j) {
        float th = o_det_theta(j), ux = sinf(th), uy = cosf(th);
        float den = vx * ux + vy * uy;
        if (den <= 1.0e-10f) continue;
        float pdot = x * ux + y * uy;
        float t = (ring_in - pdot) / den;
        if (t <= 0.0f) continue;
        float etx = cosf(th), ety = -sinf(th);
        float hx = x + t * vx, hy = y + t * vy, hz = z + t * vz;
        float q = hx * etx + hy * ety, w = hz;
        if (q * q + w * w <= throat_r * throat_r && t < best_t) { best_t = t; best = j; }
    }
    if (best < 0) return -1;
    float th = o_det_theta(best), ux = sinf(th), uy = cosf(th), etx = cosf(th), ety = -sinf(th);
    float hx = x + best_t * vx, hy = y + best_t * vy;
    float s = ring_in, q = hx * etx + hy * ety, w = z + best_t * vz;
    float vs = vx * ux + vy * uy, vq = vx * etx + vy * ety, vw = vz;
    int interactions = 0, reflections = 0;
    if (!o_bore_segment(st, model, n_air, n_bore, max_bounces, throat_out, throat_r, &s, &q, &w, &vs, &vq, &vw,
                        &interactions, &reflections))
        return -1;
    if (!o_bore_segment(st, model, n_air, n_bore, max_bounces, ring_out, counterbore_r, &s, &q, &w, &vs, &vq, &vw,
                        &interactions, &reflections))
        return -1;
    *bounce_count = reflections;
    return best;
}

/* ---------------- complex-index particle interface (:1377-1453) ---------------- */
typedef struct { float re, im; } o_cpx;
static inline o_cpx o_c(float re, float im) { o_cpx z; z.re = re; z.im = im; return z; }
static inline o_cpx o_cadd(o_cpx a, o_cpx b) { return o_c(a.re + b.re, a.im + b.im); }
static inline o_cpx o_csub(o_cpx a, o_cpx b) { return o_c(a.re - b.re, a.im - b.im); }
static inline o_cpx o_cmul(o_cpx a, o_cpx b) { return o_c(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
static inline o_cpx o_cdiv(o_cpx a, o_cpx b) {
    float d = b.re * b.re + b.im * b.im;
    if (d < 1e-30f) d = 1e-30f;
    return o_c((a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d);
}
static inline float o_cabs2(o_cpx a) { return a.re * a.re + a.im * a.im; }
static inline o_cpx o_csqrtp(o_cpx z) {
    float r = sqrtf(z.re * z.re + z.im * z.im);
    float u = sqrtf(fmaxf(0.0f, 0.5f * (r + z.re)));
    float v = sqrtf(fmaxf(0.0f, 0.5f * (r - z.re)));
    if (z.im < 0.0f) v = -v;
    if (u < 0.0f || (fabsf(u) < 1e-20f && v < 0.0f)) { u = -u; v = -v; }
    return o_c(u, v);
}
static int o_particle_interface(float ci, float n1r, float n1k, float n2r, float n2k, float* reflected,
                                float* tangential, float* normal) {
    if (!(n1r > 0.f && n2r > 0.f && n1k >= 0.f && n2k >= 0.f)) return 0;
    ci = fminf(fmaxf(ci, 0.f), 1.f);
    float beta = n1r * sqrtf(fmaxf(0.f, 1.f - ci * ci));
    o_cpx n1 = o_c(n1r, n1k), n2 = o_c(n2r, n2k);
    o_cpx eps1 = o_cmul(n1, n1), eps2 = o_cmul(n2, n2);
    o_cpx q1 = o_csqrtp(o_csub(eps1, o_c(beta * beta, 0.f)));
    o_cpx q2 = o_csqrtp(o_csub(eps2, o_c(beta * beta, 0.f)));
    o_cpx rs = o_cdiv(o_csub(q1, q2), o_cadd(q1, q2));
    o_cpx rp = o_cdiv(o_csub(o_cmul(eps2, q1), o_cmul(eps1, q2)), o_cadd(o_cmul(eps2, q1), o_cmul(eps1, q2)));
    float R = .5f * (o_cabs2(rs) + o_cabs2(rp));
    if (!isfinite(R)) return 0;
    o_cpx qeps = o_cdiv(q2, eps2), beps = o_cdiv(o_c(beta, 0.f), eps2);
    float Sx = beta, Sz = q2.re, Px = beps.re, Pz = qeps.re;
    float sn = hypotf(Sx, Sz), pn = hypotf(Px, Pz);
    if (!(sn > 0.f && pn > 0.f && Sz >= 0.f && Pz >= 0.f)) return 0;
    float txe = .5f * (Sx / sn + Px / pn);
    float tze = .5f * (Sz / sn + Pz / pn);
    float nm = hypotf(txe, tze);
    if (!(nm > 0.f && isfinite(nm))) return 0;
    *reflected = fminf(fmaxf(R, 0.f), 1.f);
    *tangential = txe / nm;
    *normal = tze / nm;
    return 1;
}
static int o_particle_refract(float ix, float iy, float iz, float nx, float ny, float nz, float n1r, float n1k,
                              float n2r, float n2k, float* ox, float* oy, float* oz) {
    float ci = fminf(fmaxf(-o_dot(ix, iy, iz, nx, ny, nz), 0.f), 1.f);
    float R, ts, tn;
    if (!o_particle_interface(ci, n1r, n1k, n2r, n2k, &R, &ts, &tn)) return 0;
    float px = ix + ci * nx, py = iy + ci * ny, pz = iz + ci * nz;
    float pn = sqrtf(px * px + py * py + pz * pz);
    if (pn > 1.e-7f) { px /= pn; py /= pn; pz /= pn; }
    else { px = py = pz = 0.f; ts = 0.f; tn = 1.f; }
    *ox = ts * px - tn * nx; *oy = ts * py - tn * ny; *oz = ts * pz - tn * nz;
    o_normalize(ox, oy, oz);
    return isfinite(*ox) && isfinite(*oy) && isfinite(*oz);
}

/* ---------------- free surfaces (:1503-1527, :1611-1779) ---------------- */
static inline float o_scully_hinf(float R, float dh, float core) {
    float a2 = core * core, R2 = R * R;
    return dh * (a2 + R2) / R2;
}
static inline float o_scully_hbar(float R, float dh, float core) {
    float a2 = core * core, R2 = R * R;
    float H = o_scully_hinf(R, dh, core);
    return H * (1.0f - (a2 / R2) * log1pf(R2 / a2));
}
/* Rankine vortex surface (model 3): new in this library, no reference lines to follow. Solid-body core
 * r <= a and free vortex outside: z0 + k r^2 inside, z0 + k a^2 (2 - a^2/r^2) outside, with
 * k = dh / (a^2 (2 - a^2/R^2)) and z0 = zmean - (k/R^2)(a^4/2 + 2 a^2 (R^2 - a^2) - 2 a^4 ln(R/a)) (volume
 * conservation); a core wider than the tube is clamped to it. FP64 coefficients. */
static inline void o_rankine(double zmean, double R, double dh, double core, double* k, double* a2, double* z0) {
    double R2 = R * R, a = fmin(core, R);
    *a2 = a * a;
    *k = dh / (*a2 * (2.0 - *a2 / R2));
    *z0 = zmean - (*k / R2) * (0.5 * *a2 * *a2 + 2.0 * *a2 * (R2 - *a2) - 2.0 * *a2 * *a2 * log(R / a));
}
static inline double o_rankine_z(double k, double a2, double z0, double q) {
    return (q <= a2) ? z0 + k * q : z0 + k * a2 * (2.0 - a2 / q);
}
static inline float o_surface_z(float x, float y, float zmean, float R, int model, float dh, float core) {
    if (model == 0 || dh <= 0.0f) return zmean;
    float q = x * x + y * y;
    if (model == 1) return zmean + dh * (q / (R * R) - 0.5f);
    if (model == 3) {
        double k, a2, z0;
        o_rankine(zmean, R, dh, core, &k, &a2, &z0);
        return (float)o_rankine_z(k, a2, z0, (double)q);
    }
    float a2 = core * core;
    float H = o_scully_hinf(R, dh, core);
    float hbar = o_scully_hbar(R, dh, core);
    return zmean - hbar + H * q / (a2 + q);
}
static double o_quadratic_min_positive(double A, double B, double Cc) {
    const double eps = 0.0;
    if (fabs(A) < 1e-24) {
        if (fabs(B) < 1e-24) return 1.0e300;
        double t = -Cc / B;
        return t > eps ? t : 1.0e300;
    }
    double D = B * B - 4.0 * A * Cc;
    if (D < 0.0) return 1.0e300;
    double sd = sqrt(fmax(D, 0.0));
    double q = -0.5 * (B + copysign(sd, B));
    double t1 = (fabs(q) > 1e-300) ? q / A : (-B - sd) / (2.0 * A);
    double t2 = (fabs(q) > 1e-300) ? Cc / q : (-B + sd) / (2.0 * A);
    double best = 1.0e300;
    if (t1 > eps && t1 < best) best = t1;
    if (t2 > eps && t2 < best) best = t2;
    return best;
}
static double o_cubic_min_positive(double A3, double A2, double A1, double A0) {
    const double eps = 0.0;
    double scale = fmax(fmax(fabs(A3), fabs(A2)), fmax(fabs(A1), fabs(A0)));
    if (scale <= 0.0) return 1.0e300;
    if (fabs(A3) <= 1e-12) return o_quadratic_min_positive(A2, A1, A0);
    double a = A2 / A3, b = A1 / A3, c = A0 / A3;
    double p = b - a * a / 3.0;
    double q = 2.0 * a * a * a / 27.0 - a * b / 3.0 + c;
    double halfq = 0.5 * q, thirdp = p / 3.0;
    double d1 = halfq * halfq, d2 = thirdp * thirdp * thirdp;
    double disc = d1 + d2;
    double tol = 1e-12 * (fabs(d1) + fabs(d2) + 1e-300);
    double best = 1.0e300;
    if (disc > tol) {
        double sd = sqrt(disc);
        double u = cbrt(-halfq + sd), v = cbrt(-halfq - sd);
        double t = u + v - a / 3.0;
        if (t > eps) best = t;
    } else if (fabs(p) < 1e-24 && fabs(q) < 1e-24) {
        double t = -a / 3.0;
        if (t > eps) best = t;
    } else if (disc >= -tol) {
        double u = cbrt(-halfq);
        double t1 = 2.0 * u - a / 3.0;
        double t2 = -u - a / 3.0;
        if (t1 > eps && t1 < best) best = t1;
        if (t2 > eps && t2 < best) best = t2;
    } else {
        double m = 2.0 * sqrt(fmax(-thirdp, 0.0));
        double den = sqrt(fmax(-(thirdp * thirdp * thirdp), 1e-300));
        double ca = fmin(fmax(-halfq / den, -1.0), 1.0);
        double phi = acos(ca);
        for (int k = 0; k < 3; ++k) {
            double t = m * cos((phi + 2.0 * O_PI_D * (double)k) / 3.0) - a / 3.0;
            if (t > eps && t < best) best = t;
        }
    }
    return best;
}
static double o_scully_bounded_root(double a3, double a2, double a1, double a0, double lo, double hi) {
    if (!(hi > lo) || !isfinite(hi)) return 1.0e300;
    double cuts[4];
    int n = 1;
    cuts[0] = lo;
    double A = 3.0 * a3, B = 2.0 * a2, Cc = a1;
    if (A != 0.0) {
        double disc = B * B - 4.0 * A * Cc;
        if (disc >= 0.0) {
            double q = -0.5 * (B + copysign(sqrt(disc), B));
            double r1 = (q != 0.0) ? q / A : -B / (2.0 * A);
            double r2 = (q != 0.0) ? Cc / q : r1;
            if (r1 > lo && r1 < hi) cuts[n++] = r1;
            if (r2 > lo && r2 < hi && r2 != r1) cuts[n++] = r2;
        }
    } else if (B != 0.0) {
        double r = -Cc / B;
        if (r > lo && r < hi) cuts[n++] = r;
    }
    cuts[n++] = hi;
    for (int i = 1; i < n; ++i) {
        double v = cuts[i];
        int j = i;
        while (j > 0 && cuts[j - 1] > v) { cuts[j] = cuts[j - 1]; --j; }
        cuts[j] = v;
    }
    for (int i = 0; i < n - 1; ++i) {
        double l = cuts[i], r = cuts[i + 1];
        double fl = ((a3 * l + a2) * l + a1) * l + a0;
        double fr = ((a3 * r + a2) * r + a1) * r + a0;
        if (l > 0.0 && fl == 0.0) return l;
        if ((fl < 0.0 && fr > 0.0) || (fl > 0.0 && fr < 0.0)) {
            for (int j = 0; j < 64; ++j) {
                double m = l + 0.5 * (r - l);
                if (m == l || m == r) break;
                double fm = ((a3 * m + a2) * m + a1) * m + a0;
                if (fm == 0.0) { l = r = m; break; }
                if ((fl < 0.0 && fm < 0.0) || (fl > 0.0 && fm > 0.0)) { l = m; fl = fm; }
                else r = m;
            }
            return l + 0.5 * (r - l);
        }
        if (r > 0.0 && fr == 0.0) return r;
    }
    return 1.0e300;
}
/* Rankine surface crossing (model 3, new): the ray's chord inside the tube split where it crosses the core
 * cylinder; on each piece the first sign change of z(t) - zs(t) (a quadratic inside the core, the cubic
 * q(t)(z(t) - z0 - 2 k a^2) + k a^4 outside) by the bounded-root search. */
static float o_rankine_hit(float x, float y, float z, float vx, float vy, float vz, float zmean, float R, float dh,
                           float core) {
    double k, a2, z0;
    o_rankine(zmean, R, dh, core, &k, &a2, &z0);
    double X = x, Y = y, Z = z, VX = vx, VY = vy, VZ = vz, RR = (double)R * (double)R;
    double Q2 = VX * VX + VY * VY, Q1 = 2.0 * (X * VX + Y * VY), Q0 = X * X + Y * Y;
    if (!(Q2 > 0.0)) {
        double t = (VZ != 0.0) ? (o_rankine_z(k, a2, z0, Q0) - Z) / VZ : 1.0e300;
        return (t > 0.0 && Q0 <= RR * (1.0 + 2e-6) && t < 0.5 * (double)O_INF_F) ? (float)t : O_INF_F;
    }
    double dc = Q1 * Q1 - 4.0 * Q2 * (Q0 - RR);
    if (dc < 0.0) return O_INF_F;
    double q = -0.5 * (Q1 + copysign(sqrt(dc), Q1));
    double ta = (q != 0.0) ? q / Q2 : -Q1 / (2.0 * Q2), tb = (q != 0.0) ? (Q0 - RR) / q : ta;
    double lo = fmax(0.0, fmin(ta, tb)), hi = fmax(ta, tb);
    if (!(hi > lo)) return O_INF_F;
    double cuts[4];
    int n = 0;
    cuts[n++] = lo;
    double dcore = Q1 * Q1 - 4.0 * Q2 * (Q0 - a2);
    if (dcore > 0.0) {
        q = -0.5 * (Q1 + copysign(sqrt(dcore), Q1));
        ta = (q != 0.0) ? q / Q2 : -Q1 / (2.0 * Q2);
        tb = (q != 0.0) ? (Q0 - a2) / q : ta;
        double c1 = fmin(ta, tb), c2 = fmax(ta, tb);
        if (c1 > lo && c1 < hi) cuts[n++] = c1;
        if (c2 > lo && c2 < hi && c2 > c1) cuts[n++] = c2;
    }
    cuts[n++] = hi;
    for (int i = 0; i < n - 1; ++i) {
        double l = cuts[i], r = cuts[i + 1], m = 0.5 * (l + r), t;
        double qm = Q0 + m * (Q1 + m * Q2);
        if (qm <= a2) {
            t = o_scully_bounded_root(0.0, -k * Q2, VZ - k * Q1, Z - z0 - k * Q0, l, r);
        } else {
            double L = Z - z0 - 2.0 * k * a2;
            t = o_scully_bounded_root(VZ * Q2, L * Q2 + VZ * Q1, L * Q1 + VZ * Q0, L * Q0 + k * a2 * a2, l, r);
        }
        if (t > 0.0 && t < 0.5 * (double)O_INF_F) return (float)t;
    }
    return O_INF_F;
}
/* first positive ray/free-surface intersection (:1715-1765) */
static float o_surface_hit(float x, float y, float z, float vx, float vy, float vz, float zmean, float R, int model,
                          float dh, float core) {
    if (model == 0 || dh <= 0.0f) {
        if (fabsf(vz) <= 1e-14f) return O_INF_F;
        float t = (zmean - z) / vz;
        return (t > 0.0f) ? t : O_INF_F;
    }
    if (model == 3) return o_rankine_hit(x, y, z, vx, vy, vz, zmean, R, dh, core);
    if (model == 1) {
        float aa = dh / (R * R);
        double A = -(double)aa * ((double)vx * vx + (double)vy * vy);
        double B = (double)vz - 2.0 * (double)aa * ((double)x * vx + (double)y * vy);
        double Cc = (double)z - ((double)zmean - 0.5 * (double)dh) - (double)aa * ((double)x * x + (double)y * y);
        double t = o_quadratic_min_positive(A, B, Cc);
        return (t < 0.5 * (double)O_INF_F) ? (float)t : O_INF_F;
    }
    double X = x, Y = y, Z = z, VX = vx, VY = vy, VZ = vz;
    double RR = (double)R * (double)R, aa = (double)core * (double)core;
    double H = (double)dh * (aa + RR) / RR;
    double hbar = H * (1.0 - (aa / RR) * log1p(RR / aa));
    double Csurf = (double)zmean - hbar;
    double Q2 = VX * VX + VY * VY;
    double Q1 = 2.0 * (X * VX + Y * VY);
    double Q0 = X * X + Y * Y;
    double L0 = Z - Csurf;
    double c3 = VZ * Q2;
    double c2 = (L0 - H) * Q2 + VZ * Q1;
    double c1 = (L0 - H) * Q1 + VZ * (aa + Q0);
    double c0 = L0 * aa + (L0 - H) * Q0;
    double t = o_cubic_min_positive(c3, c2, c1, c0);
    double xx = X + t * VX, yy = Y + t * VY, qq = xx * xx + yy * yy;
    double residual = (Z + t * VZ) - (Csurf + H * qq / (aa + qq));
    double tol = 32.0 * 2.2204460492503131e-16 * fmax(fmax(fabs(Z), fabs(Csurf) + fabs(H)), 1.0e-3);
    if (!(t < 0.5 * (double)O_INF_F) || qq > RR * (1.0 + 2e-6) || !isfinite(residual) || fabs(residual) > tol) {
        if (Q2 > 0.0) {
            double dc = Q1 * Q1 - 4.0 * Q2 * (Q0 - RR);
            if (dc < 0.0) return O_INF_F;
            double q = -0.5 * (Q1 + copysign(sqrt(dc), Q1));
            double ta = (q != 0.0) ? q / Q2 : -Q1 / (2.0 * Q2);
            double tb = (q != 0.0) ? (Q0 - RR) / q : ta;
            double lo = fmax(0.0, fmin(ta, tb)), hi = fmax(ta, tb);
            t = o_scully_bounded_root(c3, c2, c1, c0, lo, hi);
        } else {
            t = (VZ != 0.0) ? ((Csurf + H * Q0 / (aa + Q0)) - Z) / VZ : 1.0e300;
            if (!(t > 0.0) || Q0 > RR * (1.0 + 2e-6)) return O_INF_F;
        }
    }
    return (t > 0.0 && t < 0.5 * (double)O_INF_F) ? (float)t : O_INF_F;
}
/* unit normal into the water (:1768-1779) */
static inline void o_surface_normal(float x, float y, float R, int model, float dh, float core, float* nx, float* ny,
                                    float* nz) {
    if (model == 0 || dh <= 0.0f) { *nx = 0.0f; *ny = 0.0f; *nz = -1.0f; return; }
    if (model == 1) {
        float aa = dh / (R * R);
        *nx = 2.0f * aa * x; *ny = 2.0f * aa * y; *nz = -1.0f;
        o_normalize(nx, ny, nz);
        return;
    }
    if (model == 3) {  /* dz/dr = 2 k r in the core, 2 k a^4 / r^3 outside */
        double k, ra2, z0, qq = (double)x * x + (double)y * y;
        o_rankine(0.0, R, dh, core, &k, &ra2, &z0);
        float fac = (float)((qq <= ra2) ? 2.0 * k : 2.0 * k * ra2 * ra2 / (qq * qq));
        *nx = fac * x; *ny = fac * y; *nz = -1.0f;
        o_normalize(nx, ny, nz);
        return;
    }
    float a2 = core * core, q = x * x + y * y;
    float H = o_scully_hinf(R, dh, core);
    float fac = 2.0f * H * a2 / ((a2 + q) * (a2 + q));
    *nx = fac * x; *ny = fac * y; *nz = -1.0f;
    o_normalize(nx, ny, nz);
}
static inline void o_perp_basis(float vx, float vy, float vz, float* e1x, float* e1y, float* e1z, float* e2x,
                                float* e2y, float* e2z) {
    float rx, ry, rz;
    if (fabsf(vy) < 0.9f) { rx = 0.0f; ry = 1.0f; rz = 0.0f; }
    else { rx = 1.0f; ry = 0.0f; rz = 0.0f; }
    *e1x = ry * vz - rz * vy; *e1y = rz * vx - rx * vz; *e1z = rx * vy - ry * vx;
    o_normalize(e1x, e1y, e1z);
    *e2x = vy * (*e1z) - vz * (*e1y); *e2y = vz * (*e1x) - vx * (*e1z); *e2z = vx * (*e1y) - vy * (*e1x);
    o_normalize(e2x, e2y, e2z);
}

/* ---------------- sediment field lookup (:1537-1609) ---------------- */
typedef struct {
    int model, surface_model, n_bins, n_radial, grid_nr, grid_nz;
    const double *A, *B, *norm, *radial_log, *grid;
    float grid_zmax, R, zmin, core;
} o_field;

static double o_grid_sample(const o_field* f, int pidx, float x, float y, float z) {
    const int NR = f->grid_nr, NZ = f->grid_nz;
    if (NR < 2 || NZ < 2 || !(f->grid_zmax > f->zmin)) return 1.0;
    double rr = sqrt(fmax((double)x * (double)x + (double)y * (double)y, 0.0));
    if (rr < 0.0) rr = 0.0;
    if (rr > (double)f->R) rr = (double)f->R;
    double dr = (double)f->R / (double)NR, dz = ((double)f->grid_zmax - (double)f->zmin) / (double)NZ;
    double ur = rr / dr - 0.5, uz = ((double)z - (double)f->zmin) / dz - 0.5;
    if (ur < 0.0) ur = 0.0;
    if (uz < 0.0) uz = 0.0;
    if (ur > (double)(NR - 1)) ur = (double)(NR - 1);
    if (uz > (double)(NZ - 1)) uz = (double)(NZ - 1);
    int i = (int)floor(ur), k = (int)floor(uz);
    double tr = ur - (double)i, tz = uz - (double)k;
    if (i >= NR - 1) { i = NR - 2; tr = 1.0; }
    if (k >= NZ - 1) { k = NZ - 2; tz = 1.0; }
    long long plane = (long long)NR * (long long)NZ;
    long long b = (long long)pidx * plane;
    const double* G = f->grid;
    double q00 = G[b + (long long)i * NZ + k];
    double q10 = G[b + (long long)(i + 1) * NZ + k];
    double q01 = G[b + (long long)i * NZ + k + 1];
    double q11 = G[b + (long long)(i + 1) * NZ + k + 1];
    double q0 = (1.0 - tr) * q00 + tr * q10, q1 = (1.0 - tr) * q01 + tr * q11;
    return fmax((1.0 - tz) * q0 + tz * q1, 0.0);
}
static double o_local_scale(const o_field* f, int pidx, float x, float y, float z) {
    if (f->model == 0) return 1.0;
    if (f->model == 3) return o_grid_sample(f, pidx, x, y, z);
    const float R = f->R;
    double rr2 = (double)x * (double)x + (double)y * (double)y;
    double R2 = (double)R * (double)R;
    if (rr2 > R2) rr2 = R2;
    double radial_log = 0.0;
    if (f->model == 1) {
        if (f->surface_model == 1) {
            radial_log = f->A[pidx] * (rr2 - R2);
        } else {
            double a2 = (double)f->core * (double)f->core;
            double fr = rr2 / (a2 + rr2), fR = R2 / (a2 + R2);
            radial_log = f->A[pidx] * (fr - fR);
        }
    } else {
        double rr = sqrt(fmax(rr2, 0.0));
        double u = (R > 0.0) ? rr / (double)R * (double)(f->n_radial - 1) : 0.0;
        int j = (int)floor(u);
        if (j < 0) j = 0;
        if (j > f->n_radial - 2) j = f->n_radial - 2;
        double t = u - (double)j;
        long long base = (long long)pidx * (long long)f->n_radial;
        radial_log = (1.0 - t) * f->radial_log[base + j] + t * f->radial_log[base + j + 1];
        if (radial_log > 0.0) radial_log = 0.0;
    }
    double h = fmax((double)z - (double)f->zmin, 0.0);
    double logrel = radial_log - f->B[pidx] * h;
    double ns = f->norm[pidx];
    if (!(ns > 0.0)) return 0.0;
    return exp(logrel) / ns;
}
static int o_sample_local_bin(uint32_t* s, const o_field* f, const double* mu_bin, float x, float y, float z,
                              double local_total) {
    if (!(local_total > 0.0)) return 0;
    double target = (double)o_uniform(s) * local_total, cum = 0.0;
    for (int i = 0; i < f->n_bins; ++i) {
        double sc = o_local_scale(f, i, x, y, z);
        cum += mu_bin[i] * sc;
        if (target <= cum) return i;
    }
    return f->n_bins > 0 ? f->n_bins - 1 : 0;
}

#endif
