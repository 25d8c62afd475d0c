// Device physics, part A: samplers, ray optics, collimator bores, complex-index
// interfaces, free surfaces, sediment field lookup and polynomial roots.
//
// Each function restates the reference device function named beside it (file
// CLARITAS/CLARITAS.py) with the same floating-point operation order: in the
// reference's xorshift mode the kernel reproduces the reference's per-ray
// integer outcomes exactly on the same GPU (tests/test_gpu_parity.py).
// Functions take the random stream as a template parameter so the same code
// serves the xorshift parity streams and the Philox production stream.
#pragma once
#include <cstdint>
#include "rng.cuh"

#define CLR_INF_F 3.402823466e+38F
#define CLR_PI_F 3.14159265358979323846f
#define CLR_EPS_F 2.0e-7f
#define CLR_PI_D 3.141592653589793238462643383279502884
#define CLR_DBL_EPS 2.220446049250313080847263336181640625e-16

namespace clr {
namespace {  // header-only device code: internal linkage in every translation unit
/* ---------------- samplers (:1148-1212) ---------------- */
template <class S>
__device__ __forceinline__ float o_normal(S* s) {
    float u1 = fmaxf(uniform(s), 1e-12f), u2 = uniform(s);
    return sqrtf(-2.0f * logf(u1)) * cosf(2.0f * CLR_PI_F * u2);
}
template <class S>
__device__ float o_gamma(S* s, float shape) {
    if (shape <= 0.0f) return 0.0f;
    if (fabsf(shape - 1.0f) < 1e-7f) return -logf(fmaxf(uniform(s), 1e-12f));
    float correction = 1.0f, a = shape;
    if (a < 1.0f) {
        float u = fmaxf(uniform(s), 1e-12f);
        correction = powf(u, 1.0f / a);
        a += 1.0f;
    }
    float d = a - 0.3333333333333333f;
    float c = rsqrtf(9.0f * d);
    for (int it = 0; it < 128; ++it) {
        float x = o_normal(s);
        float v = 1.0f + c * x;
        if (v <= 0.0f) continue;
        v = v * v * v;
        float u = uniform(s);
        if (u < 1.0f - 0.0331f * x * x * x * x) return correction * d * v;
        if (logf(fmaxf(u, 1e-12f)) < 0.5f * x * x + d * (1.0f - v + logf(v))) return correction * d * v;
    }
    return correction * d;
}
template <class S>
__device__ float o_beta(S* s, float a, float b) {
    if (a <= 0.0f || b <= 0.0f) return 0.0f;
    if (fabsf(a - 1.0f) < 1e-7f) {
        float u = fminf(fmaxf(uniform(s), 1e-12f), 1.0f - 1e-7f);
        return 1.0f - powf(1.0f - u, 1.0f / b);
    }
    if (fabsf(b - 1.0f) < 1e-7f) {
        float u = fminf(fmaxf(uniform(s), 1e-12f), 1.0f - 1e-7f);
        return powf(u, 1.0f / a);
    }
    float ga = o_gamma(s, a), gb = o_gamma(s, b);
    float t = ga + gb;
    return t > 0.0f ? ga / t : 0.0f;
}
/* Beta angular-radiance polar angle, rejection by sin(x)/x (:1201-1212) */
template <class S>
__device__ float o_beta_radiance_polar(S* s, float a, float b) {
    const float c = 0.5f * CLR_PI_F;
    for (int it = 0; it < 128; ++it) {
        float u = o_beta(s, a + 1.0f, b);
        u = fminf(fmaxf(u, 0.0f), 1.0f);
        float x = c * u;
        float accept = (x < 1.0e-7f) ? 1.0f : sinf(x) / x;
        if (uniform(s) <= accept) return x;
    }
    float u = o_beta(s, a + 1.0f, b);
    return c * fminf(fmaxf(u, 0.0f), 1.0f);
}

/* ---------------- vectors and Fresnel (:1214-1260) ---------------- */
__device__ __forceinline__ float o_dot(float ax, float ay, float az, float bx, float by, float bz) {
    return ax * bx + ay * by + az * bz;
}
__device__ __forceinline__ void o_normalize(float* x, float* y, float* z) {
    float q = (*x) * (*x) + (*y) * (*y) + (*z) * (*z);
    if (q <= 0.0f) { *x = 0.0f; *y = 1.0f; *z = 0.0f; return; }
    float s = rsqrtf(q);
    *x *= s; *y *= s; *z *= s;
}
__device__ __forceinline__ void o_reflect(float ix, float iy, float iz, float nx, float ny, float nz, float* ox, float* oy, float* oz) {
    float d = o_dot(ix, iy, iz, nx, ny, nz);
    *ox = ix - 2.0f * d * nx; *oy = iy - 2.0f * d * ny; *oz = iz - 2.0f * d * nz;
    o_normalize(ox, oy, oz);
}
/* n points into the incident medium; returns 0 on total internal reflection */
__device__ __forceinline__ int o_refract(float ix, float iy, float iz, float nx, float ny, float nz, float n1, float n2,
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
__device__ __forceinline__ float o_fresnel(float ci, float n1, float n2, int* tir) {
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
__device__ __forceinline__ void o_radial_normal(float x, float y, float* nx, float* ny) {
    float r = sqrtf(fmaxf(x * x + y * y, 1e-30f));
    *nx = x / r; *ny = y / r;
}

/* ---------------- collimator bores (:1263-1374) ---------------- */
__device__ __forceinline__ float o_bore_side_hit(float q, float w, float vq, float vw, float radius) {
    float A = vq * vq + vw * vw;
    if (A <= 1.0e-20f) return CLR_INF_F;
    float B = 2.0f * (q * vq + w * vw);
    float Cc = q * q + w * w - radius * radius;
    float D = B * B - 4.0f * A * Cc;
    if (D < 0.0f) return CLR_INF_F;
    float root = sqrtf(fmaxf(D, 0.0f));
    float t1 = (-B - root) / (2.0f * A), t2 = (-B + root) / (2.0f * A);
    float t = CLR_INF_F;
    if (t1 > CLR_EPS_F) t = t1;
    if (t2 > CLR_EPS_F && t2 < t) t = t2;
    return t;
}
template <class S>
__device__ int o_bore_wall_reflect(S* s, int model, float n_air, float n_bore, float q, float w, float* vs,
                               float* vq, float* vw, int* interactions, int* reflections) {
    (*interactions)++;
    if (model == 0) return 0;
    float rr = sqrtf(fmaxf(q * q + w * w, 1.0e-30f));
    float ns = 0.0f, nq = -q / rr, nw = -w / rr;
    float ci = fminf(fmaxf(-((*vs) * ns + (*vq) * nq + (*vw) * nw), 0.0f), 1.0f);
    int tir = 0;
    float R = o_fresnel(ci, n_air, n_bore, &tir);
    if (uniform(s) >= R) return 0;
    float os, oq, ow;
    o_reflect(*vs, *vq, *vw, ns, nq, nw, &os, &oq, &ow);
    *vs = os; *vq = oq; *vw = ow;
    (*reflections)++;
    return 1;
}
template <class S>
__device__ __noinline__ int o_bore_segment(S* st, int model, float n_air, float n_bore, int max_bounces, float s_end,
                          float radius, float* s, float* q, float* w, float* vs, float* vq, float* vw,
                          int* interactions, int* reflections) {
    for (int b = 0; b <= max_bounces; ++b) {
        if (*vs <= 1.0e-12f) return 0;
        float tp = (s_end - *s) / (*vs);
        if (tp < -CLR_EPS_F) return 0;
        if (tp < 0.0f) tp = 0.0f;
        float twall = o_bore_side_hit(*q, *w, *vq, *vw, radius);
        if (tp <= twall) {
            *q += tp * (*vq); *w += tp * (*vw); *s = s_end;
            return ((*q) * (*q) + (*w) * (*w) <= radius * radius * (1.0f + 2.0e-5f));
        }
        if (twall >= CLR_INF_F * 0.5f) return 0;
        *q += twall * (*vq); *w += twall * (*vw); *s += twall * (*vs);
        if (!o_bore_wall_reflect(st, model, n_air, n_bore, *q, *w, vs, vq, vw, interactions, reflections)) return 0;
        float rr = sqrtf(fmaxf((*q) * (*q) + (*w) * (*w), 1.0e-30f));
        *q -= CLR_EPS_F * (*q) / rr; *w -= CLR_EPS_F * (*w) / rr;
    }
    return 0;
}
template <class S>
__device__ int o_source_collimator(S* st, int model, float n_air, float n_bore, int max_bounces, float ring_in,
                               float throat_out, float source_r, float throat_r, float counterbore_r, float* x,
                               float* y, float* z, float* vx, float* vy, float* vz, int* interactions,
                               int* reflections) {
    (void)source_r;
    if (*vy <= 1.0e-12f) return 0;
    float s = *y, q = *x, w = *z, vs = *vy, vq = *vx, vw = *vz;
    if (q * q + w * w > counterbore_r * counterbore_r) return 0;
    float shoulder = -throat_out;
    if (s < shoulder - CLR_EPS_F) {
        if (!o_bore_segment(st, model, n_air, n_bore, max_bounces, shoulder, counterbore_r, &s, &q, &w, &vs, &vq, &vw,
                            interactions, reflections))
            return 0;
    } else if (s > shoulder + CLR_EPS_F) {
        return 0;
    }
    if (q * q + w * w > throat_r * throat_r) return 0;
    if (!o_bore_segment(st, model, n_air, n_bore, max_bounces, -ring_in, throat_r, &s, &q, &w, &vs, &vq, &vw,
                        interactions, reflections))
        return 0;
    *x = q; *y = s; *z = w; *vx = vq; *vy = vs; *vz = vw;
    return 1;
}
/* bore directions: sin/cos of (10 j)(pi/180), j = 0..18 (the 18 detectors and the source bore). The kernel
 * evaluates them once per block with the same device sinf/cosf the reference calls per use (:4241-4244),
 * so the table holds exactly the values the reference recomputes. */
__device__ __forceinline__ float o_det_theta(int j) { return (10.0f * (float)j) * (CLR_PI_F / 180.0f); }

template <class S>
__device__ __noinline__ int o_detector_collimator_path(S* st, float x, float y, float z, float vx, float vy, float vz,
                                      int mirror, float ring_in, float throat_out, float ring_out, float throat_r,
                                      float counterbore_r, int model, float n_air, float n_bore, int max_bounces,
                                      int* bounce_count, const float* dsin, const float* dcos) {
    if (mirror) { x = -x; vx = -vx; }
    float best_t = CLR_INF_F;
    int best = -1;
    for (int j = 0; j < 18; ++j) {
        float ux = dsin[j], uy = dcos[j];
        float den = vx * ux + vy * uy;
        if (den <= 1.0e-10f) continue;
        float pdot = x * ux + y * uy;
        float t = (ring_in - pdot) / den;
        if (t <= 0.0f) continue;
        float etx = dcos[j], ety = -dsin[j];
        float hx = x + t * vx, hy = y + t * vy, hz = z + t * vz;
        float q = hx * etx + hy * ety, w = hz;
        if (q * q + w * w <= throat_r * throat_r && t < best_t) { best_t = t; best = j; }
    }
    if (best < 0) return -1;
    float ux = dsin[best], uy = dcos[best], etx = dcos[best], ety = -dsin[best];
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
__device__ __forceinline__ o_cpx o_c(float re, float im) { o_cpx z; z.re = re; z.im = im; return z; }
__device__ __forceinline__ o_cpx o_cadd(o_cpx a, o_cpx b) { return o_c(a.re + b.re, a.im + b.im); }
__device__ __forceinline__ o_cpx o_csub(o_cpx a, o_cpx b) { return o_c(a.re - b.re, a.im - b.im); }
__device__ __forceinline__ o_cpx o_cmul(o_cpx a, o_cpx b) { return o_c(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
__device__ __forceinline__ o_cpx o_cdiv(o_cpx a, o_cpx b) {
    float d = b.re * b.re + b.im * b.im;
    if (d < 1e-30f) d = 1e-30f;
    return o_c((a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d);
}
__device__ __forceinline__ float o_cabs2(o_cpx a) { return a.re * a.re + a.im * a.im; }
__device__ __forceinline__ o_cpx o_csqrtp(o_cpx z) {
    float r = sqrtf(z.re * z.re + z.im * z.im);
    float u = sqrtf(fmaxf(0.0f, 0.5f * (r + z.re)));
    float v = sqrtf(fmaxf(0.0f, 0.5f * (r - z.re)));
    if (z.im < 0.0f) v = -v;
    if (u < 0.0f || (fabsf(u) < 1e-20f && v < 0.0f)) { u = -u; v = -v; }
    return o_c(u, v);
}
__device__ int o_particle_interface(float ci, float n1r, float n1k, float n2r, float n2k, float* reflected,
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
__device__ int o_particle_refract(float ix, float iy, float iz, float nx, float ny, float nz, float n1r, float n1k,
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
__device__ __forceinline__ float o_scully_hinf(float R, float dh, float core) {
    float a2 = core * core, R2 = R * R;
    return dh * (a2 + R2) / R2;
}
__device__ __forceinline__ float o_scully_hbar(float R, float dh, float core) {
    float a2 = core * core, R2 = R * R;
    float H = o_scully_hinf(R, dh, core);
    return H * (1.0f - (a2 / R2) * log1pf(R2 / a2));
}
/* Rankine vortex (free-surface model 3; no reference counterpart). A stirrer turning the liquid inside
 * the core r <= a as a solid body at angular speed W and a free vortex outside (v = W a^2 / r) give, from
 * the radial pressure balance, a surface z0 + k r^2 inside and z0 + k a^2 (2 - a^2 / r^2) outside, with
 * k = W^2 / (2 g): continuous with its slope at r = a. k follows from the wall-centre height difference
 * dh = k a^2 (2 - a^2 / R^2), and z0 = zmean - hbar from volume conservation (the area mean of the surface
 * over the disc r <= R is the rest height zmean):
 *   hbar = (k / R^2) (a^4 / 2 + 2 a^2 (R^2 - a^2) - 2 a^4 ln(R / a)).
 * A core at least as wide as the tube is a solid-body (parabolic) surface. Heights are functions of
 * q = r^2, so every caller works with q. */
struct RankineF {
    float k, a2, z0;
};
__device__ __forceinline__ RankineF f_rankine(float zmean, float R, float dh, float core) {
    const float R2 = R * R, a = fminf(core, R), a2 = a * a;
    const float k = dh / (a2 * (2.0f - a2 / R2));
    const float hbar = (k / R2) * (0.5f * a2 * a2 + 2.0f * a2 * (R2 - a2) - 2.0f * a2 * a2 * logf(R / a));
    RankineF g = {k, a2, zmean - hbar};
    return g;
}
__device__ __forceinline__ float f_rankine_z(const RankineF& g, float q) {
    return (q <= g.a2) ? g.z0 + g.k * q : g.z0 + g.k * g.a2 * (2.0f - g.a2 / q);
}
struct RankineD {
    double k, a2, z0;
};
__device__ __forceinline__ RankineD d_rankine(double zmean, double R, double dh, double core) {
    const double R2 = R * R, a = fmin(core, R), a2 = a * a;
    const double k = dh / (a2 * (2.0 - a2 / R2));
    const double hbar = (k / R2) * (0.5 * a2 * a2 + 2.0 * a2 * (R2 - a2) - 2.0 * a2 * a2 * log(R / a));
    RankineD g = {k, a2, zmean - hbar};
    return g;
}
__device__ __forceinline__ double d_rankine_z(const RankineD& g, double q) {
    return (q <= g.a2) ? g.z0 + g.k * q : g.z0 + g.k * g.a2 * (2.0 - g.a2 / q);
}

__device__ __forceinline__ float o_surface_z(float x, float y, float zmean, float R, int model, float dh, float core) {
    if (model == 0 || dh <= 0.0f) return zmean;
    float q = x * x + y * y;
    if (model == 1) return zmean + dh * (q / (R * R) - 0.5f);
    if (model == 3) return f_rankine_z(f_rankine(zmean, R, dh, core), q);
    float a2 = core * core;
    float H = o_scully_hinf(R, dh, core);
    float hbar = o_scully_hbar(R, dh, core);
    return zmean - hbar + H * q / (a2 + q);
}
__device__ double o_quadratic_min_positive(double A, double B, double Cc) {
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
__device__ __noinline__ double o_cubic_min_positive(double A3, double A2, double A1, double A0) {
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
            double t = m * cos((phi + 2.0 * CLR_PI_D * (double)k) / 3.0) - a / 3.0;
            if (t > eps && t < best) best = t;
        }
    }
    return best;
}
__device__ __noinline__ double o_scully_bounded_root(double a3, double a2, double a1, double a0, double lo, double hi) {
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
/* first positive ray/free-surface intersection (:1715-1765) */
/* Rankine surface crossing (FP64): the ray's chord inside the tube is split where it crosses the core
 * cylinder q(t) = a^2; on a piece inside the core the crossing solves the quadratic z(t) - z0 - k q(t) = 0,
 * outside it the cubic q(t) (z(t) - z0 - 2 k a^2) + k a^4 = 0 (q > 0 there, so the sign is that of
 * z(t) - zs: negative below the surface). The first sign change is found by the bounded-root search. */
__device__ __noinline__ float o_rankine_hit(float x, float y, float z, float vx, float vy, float vz, float zmean,
                                           float R, float dh, float core) {
    const RankineD g = d_rankine(zmean, R, dh, core);
    const double X = x, Y = y, Z = z, VX = vx, VY = vy, VZ = vz, RR = (double)R * (double)R;
    const double Q2 = VX * VX + VY * VY, Q1 = 2.0 * (X * VX + Y * VY), Q0 = X * X + Y * Y;
    if (!(Q2 > 0.0)) {
        const double t = (VZ != 0.0) ? (d_rankine_z(g, Q0) - Z) / VZ : 1.0e300;
        return (t > 0.0 && Q0 <= RR * (1.0 + 2e-6) && t < 0.5 * (double)CLR_INF_F) ? (float)t : CLR_INF_F;
    }
    const double dc = Q1 * Q1 - 4.0 * Q2 * (Q0 - RR);
    if (dc < 0.0) return CLR_INF_F;
    double q = -0.5 * (Q1 + copysign(sqrt(dc), Q1));
    double ta = (q != 0.0) ? q / Q2 : -Q1 / (2.0 * Q2), tb = (q != 0.0) ? (Q0 - RR) / q : ta;
    const double lo = fmax(0.0, fmin(ta, tb)), hi = fmax(ta, tb);
    if (!(hi > lo)) return CLR_INF_F;
    double cuts[4];
    int n = 0;
    cuts[n++] = lo;
    const double dcore = Q1 * Q1 - 4.0 * Q2 * (Q0 - g.a2);
    if (dcore > 0.0) {
        q = -0.5 * (Q1 + copysign(sqrt(dcore), Q1));
        ta = (q != 0.0) ? q / Q2 : -Q1 / (2.0 * Q2);
        tb = (q != 0.0) ? (Q0 - g.a2) / q : ta;
        const double c1 = fmin(ta, tb), c2 = fmax(ta, tb);
        if (c1 > lo && c1 < hi) cuts[n++] = c1;
        if (c2 > lo && c2 < hi && c2 > c1) cuts[n++] = c2;
    }
    cuts[n++] = hi;
    for (int i = 0; i < n - 1; ++i) {
        const double l = cuts[i], r = cuts[i + 1], m = 0.5 * (l + r);
        const double qm = Q0 + m * (Q1 + m * Q2);
        double t;
        if (qm <= g.a2) {
            t = o_scully_bounded_root(0.0, -g.k * Q2, VZ - g.k * Q1, Z - g.z0 - g.k * Q0, l, r);
        } else {
            const double L = Z - g.z0 - 2.0 * g.k * g.a2;
            t = o_scully_bounded_root(VZ * Q2, L * Q2 + VZ * Q1, L * Q1 + VZ * Q0, L * Q0 + g.k * g.a2 * g.a2, l, r);
        }
        if (t > 0.0 && t < 0.5 * (double)CLR_INF_F) return (float)t;
    }
    return CLR_INF_F;
}
__device__ __noinline__ float o_surface_hit_curved(float x, float y, float z, float vx, float vy, float vz, float zmean,
                                                 float R, int model, float dh, float core) {
    if (model == 3) return o_rankine_hit(x, y, z, vx, vy, vz, zmean, R, dh, core);
    if (model == 1) {
        float aa = dh / (R * R);
        double A = -(double)aa * ((double)vx * vx + (double)vy * vy);
        double B = (double)vz - 2.0 * (double)aa * ((double)x * vx + (double)y * vy);
        double Cc = (double)z - ((double)zmean - 0.5 * (double)dh) - (double)aa * ((double)x * x + (double)y * y);
        double t = o_quadratic_min_positive(A, B, Cc);
        return (t < 0.5 * (double)CLR_INF_F) ? (float)t : CLR_INF_F;
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
    if (!(t < 0.5 * (double)CLR_INF_F) || qq > RR * (1.0 + 2e-6) || !isfinite(residual) || fabs(residual) > tol) {
        if (Q2 > 0.0) {
            double dc = Q1 * Q1 - 4.0 * Q2 * (Q0 - RR);
            if (dc < 0.0) return CLR_INF_F;
            double q = -0.5 * (Q1 + copysign(sqrt(dc), Q1));
            double ta = (q != 0.0) ? q / Q2 : -Q1 / (2.0 * Q2);
            double tb = (q != 0.0) ? (Q0 - RR) / q : ta;
            double lo = fmax(0.0, fmin(ta, tb)), hi = fmax(ta, tb);
            t = o_scully_bounded_root(c3, c2, c1, c0, lo, hi);
        } else {
            t = (VZ != 0.0) ? ((Csurf + H * Q0 / (aa + Q0)) - Z) / VZ : 1.0e300;
            if (!(t > 0.0) || Q0 > RR * (1.0 + 2e-6)) return CLR_INF_F;
        }
    }
    return (t > 0.0 && t < 0.5 * (double)CLR_INF_F) ? (float)t : CLR_INF_F;
}
__device__ __forceinline__ float o_surface_hit(float x, float y, float z, float vx, float vy, float vz, float zmean,
                                              float R, int model, float dh, float core) {
    if (model == 0 || dh <= 0.0f) {
        if (fabsf(vz) <= 1e-14f) return CLR_INF_F;
        float t = (zmean - z) / vz;
        return (t > 0.0f) ? t : CLR_INF_F;
    }
    return o_surface_hit_curved(x, y, z, vx, vy, vz, zmean, R, model, dh, core);
}
/* FP32 first positive crossing of the free surface, for the counter-based stream. Parabolic: the
 * quadratic by the cancellation-free formula. Scully: with q(t) = r(t)^2 the crossing solves
 * P(t) = (a^2 + q) (z(t) - zs(r(t))) = c3 t^3 + c2 t^2 + c1 t + c0 = 0 (P < 0 below the surface),
 * restricted to the chord of the ray inside the tube, where the surface formula holds: the chord is
 * split at the cubic's turning points and the first sign change is bisected to FP32 resolution. This
 * is the reference's bounded-root search (o_scully_bounded_root), which it uses whenever its Cardano
 * root fails validation; the roots agree to FP32 rounding. */
__device__ __forceinline__ float f_quadratic_min_positive(float A, float B, float Cc) {
    if (fabsf(A) < 1e-24f) {
        if (fabsf(B) < 1e-24f) return CLR_INF_F;
        const float t = -Cc / B;
        return t > 0.0f ? t : CLR_INF_F;
    }
    const float D = B * B - 4.0f * A * Cc;
    if (D < 0.0f) return CLR_INF_F;
    const float sd = sqrtf(fmaxf(D, 0.0f));
    const float q = -0.5f * (B + copysignf(sd, B));
    const float t1 = (fabsf(q) > 1e-30f) ? q / A : (-B - sd) / (2.0f * A);
    const float t2 = (fabsf(q) > 1e-30f) ? Cc / q : (-B + sd) / (2.0f * A);
    float best = CLR_INF_F;
    if (t1 > 0.0f && t1 < best) best = t1;
    if (t2 > 0.0f && t2 < best) best = t2;
    return best;
}
__device__ __forceinline__ float f_cubic(float c3, float c2, float c1, float c0, float t) {
    return ((c3 * t + c2) * t + c1) * t + c0;
}
/* First sign change of the polynomial c3 t^3 + c2 t^2 + c1 t + c0 on (l, r], FP32: the piece is split at
 * the polynomial's turning points and the first bracketing sub-piece bisected to FP32 resolution. */
__device__ float f_first_poly_root(float c3, float c2, float c1, float c0, float l0, float r0) {
    if (!(r0 > l0)) return CLR_INF_F;
    float cuts[4];
    int n = 0;
    cuts[n++] = l0;
    const float A = 3.0f * c3, B = 2.0f * c2, Cd = c1;
    if (A != 0.0f) {
        const float disc = B * B - 4.0f * A * Cd;
        if (disc >= 0.0f) {
            const float q = -0.5f * (B + copysignf(sqrtf(disc), B));
            const float r1 = (q != 0.0f) ? q / A : -B / (2.0f * A);
            const float r2 = (q != 0.0f) ? Cd / q : r1;
            const float s1 = fminf(r1, r2), s2 = fmaxf(r1, r2);
            if (s1 > l0 && s1 < r0) cuts[n++] = s1;
            if (s2 > l0 && s2 < r0 && s2 != s1) cuts[n++] = s2;
        }
    } else if (B != 0.0f) {
        const float r = -Cd / B;
        if (r > l0 && r < r0) cuts[n++] = r;
    }
    cuts[n++] = r0;
    for (int i = 0; i < n - 1; ++i) {
        float l = cuts[i], r = cuts[i + 1];
        float fl = ((c3 * l + c2) * l + c1) * l + c0;
        const float fr = ((c3 * r + c2) * r + c1) * r + c0;
        if (l > 0.0f && fl == 0.0f) return l;
        if ((fl < 0.0f && fr > 0.0f) || (fl > 0.0f && fr < 0.0f)) {
            for (int j = 0; j < 40; ++j) {
                const float m = l + 0.5f * (r - l);
                if (m == l || m == r) break;
                const float fm = ((c3 * m + c2) * m + c1) * m + c0;
                if (fm == 0.0f) { l = r = m; break; }
                if ((fl < 0.0f) == (fm < 0.0f)) { l = m; fl = fm; } else r = m;
            }
            const float t = l + 0.5f * (r - l);
            return t > 0.0f ? t : CLR_INF_F;
        }
        if (r > 0.0f && fr == 0.0f) return r;
    }
    return CLR_INF_F;
}
/* Rankine surface crossing in FP32 (counter-based stream): the pieces of o_rankine_hit. */
__device__ __noinline__ float f_rankine_hit(float x, float y, float z, float vx, float vy, float vz, float zmean,
                                            float R, float dh, float core) {
    const RankineF g = f_rankine(zmean, R, dh, core);
    const float RR = R * R;
    const float Q2 = vx * vx + vy * vy, Q1 = 2.0f * (x * vx + y * vy), Q0 = x * x + y * y;
    if (!(Q2 > 0.0f)) {
        const float t = (vz != 0.0f) ? (f_rankine_z(g, Q0) - z) / vz : CLR_INF_F;
        return (t > 0.0f && Q0 <= RR * (1.0f + 2e-6f)) ? t : CLR_INF_F;
    }
    const float dc = Q1 * Q1 - 4.0f * Q2 * (Q0 - RR);
    if (dc < 0.0f) return CLR_INF_F;
    float q = -0.5f * (Q1 + copysignf(sqrtf(dc), Q1));
    float ta = (q != 0.0f) ? q / Q2 : -Q1 / (2.0f * Q2), tb = (q != 0.0f) ? (Q0 - RR) / q : ta;
    const float lo = fmaxf(0.0f, fminf(ta, tb)), hi = fmaxf(ta, tb);
    if (!(hi > lo) || !isfinite(hi)) return CLR_INF_F;
    float cuts[4];
    int n = 0;
    cuts[n++] = lo;
    const float dcore = Q1 * Q1 - 4.0f * Q2 * (Q0 - g.a2);
    if (dcore > 0.0f) {
        q = -0.5f * (Q1 + copysignf(sqrtf(dcore), Q1));
        ta = (q != 0.0f) ? q / Q2 : -Q1 / (2.0f * Q2);
        tb = (q != 0.0f) ? (Q0 - g.a2) / q : ta;
        const float c1 = fminf(ta, tb), c2 = fmaxf(ta, tb);
        if (c1 > lo && c1 < hi) cuts[n++] = c1;
        if (c2 > lo && c2 < hi && c2 > c1) cuts[n++] = c2;
    }
    cuts[n++] = hi;
    for (int i = 0; i < n - 1; ++i) {
        const float l = cuts[i], r = cuts[i + 1], m = 0.5f * (l + r);
        const float qm = Q0 + m * (Q1 + m * Q2);
        float t;
        if (qm <= g.a2) {
            t = f_first_poly_root(0.0f, -g.k * Q2, vz - g.k * Q1, z - g.z0 - g.k * Q0, l, r);
        } else {
            const float L = z - g.z0 - 2.0f * g.k * g.a2;
            t = f_first_poly_root(vz * Q2, L * Q2 + vz * Q1, L * Q1 + vz * Q0, L * Q0 + g.k * g.a2 * g.a2, l, r);
        }
        if (t < CLR_INF_F) return t;
    }
    return CLR_INF_F;
}
__device__ __noinline__ float f_surface_hit_curved(float x, float y, float z, float vx, float vy, float vz,
                                                   float zmean, float R, int model, float dh, float core) {
    if (model == 3) return f_rankine_hit(x, y, z, vx, vy, vz, zmean, R, dh, core);
    if (model == 1) {
        const float aa = dh / (R * R);
        const float A = -aa * (vx * vx + vy * vy);
        const float B = vz - 2.0f * aa * (x * vx + y * vy);
        const float Cc = z - (zmean - 0.5f * dh) - aa * (x * x + y * y);
        return f_quadratic_min_positive(A, B, Cc);
    }
    const float RR = R * R, aa = core * core;
    const float H = dh * (aa + RR) / RR;
    const float Csurf = zmean - H * (1.0f - (aa / RR) * log1pf(RR / aa));
    const float Q2 = vx * vx + vy * vy, Q1 = 2.0f * (x * vx + y * vy), Q0 = x * x + y * y;
    const float L0 = z - Csurf;
    if (!(Q2 > 0.0f)) {  // vertical ray: the surface height is constant along it
        const float t = (vz != 0.0f) ? ((Csurf + H * Q0 / (aa + Q0)) - z) / vz : CLR_INF_F;
        return (t > 0.0f && Q0 <= RR * (1.0f + 2e-6f)) ? t : CLR_INF_F;
    }
    const float c3 = vz * Q2, c2 = (L0 - H) * Q2 + vz * Q1, c1 = (L0 - H) * Q1 + vz * (aa + Q0);
    const float c0 = L0 * aa + (L0 - H) * Q0;
    // chord of the ray inside the tube: q(t) <= R^2
    const float dc = Q1 * Q1 - 4.0f * Q2 * (Q0 - RR);
    if (dc < 0.0f) return CLR_INF_F;
    const float qq = -0.5f * (Q1 + copysignf(sqrtf(dc), Q1));
    const float ta = (qq != 0.0f) ? qq / Q2 : -Q1 / (2.0f * Q2);
    const float tb = (qq != 0.0f) ? (Q0 - RR) / qq : ta;
    const float lo = fmaxf(0.0f, fminf(ta, tb)), hi = fmaxf(ta, tb);
    if (!(hi > lo) || !isfinite(hi)) return CLR_INF_F;
    float cuts[4];
    int n = 0;
    cuts[n++] = lo;
    const float A = 3.0f * c3, B = 2.0f * c2, Cd = c1;
    if (A != 0.0f) {
        const float disc = B * B - 4.0f * A * Cd;
        if (disc >= 0.0f) {
            const float q = -0.5f * (B + copysignf(sqrtf(disc), B));
            const float r1 = (q != 0.0f) ? q / A : -B / (2.0f * A);
            const float r2 = (q != 0.0f) ? Cd / q : r1;
            const float s1 = fminf(r1, r2), s2 = fmaxf(r1, r2);
            if (s1 > lo && s1 < hi) cuts[n++] = s1;
            if (s2 > lo && s2 < hi && s2 != s1) cuts[n++] = s2;
        }
    } else if (B != 0.0f) {
        const float r = -Cd / B;
        if (r > lo && r < hi) cuts[n++] = r;
    }
    cuts[n++] = hi;
    for (int i = 0; i < n - 1; ++i) {
        float l = cuts[i], r = cuts[i + 1];
        float fl = f_cubic(c3, c2, c1, c0, l);
        const float fr = f_cubic(c3, c2, c1, c0, r);
        if (l > 0.0f && fl == 0.0f) return l;
        if ((fl < 0.0f && fr > 0.0f) || (fl > 0.0f && fr < 0.0f)) {
            for (int j = 0; j < 40; ++j) {
                const float m = l + 0.5f * (r - l);
                if (m == l || m == r) break;
                const float fm = f_cubic(c3, c2, c1, c0, m);
                if (fm == 0.0f) { l = r = m; break; }
                if ((fl < 0.0f) == (fm < 0.0f)) { l = m; fl = fm; } else r = m;
            }
            const float t = l + 0.5f * (r - l);
            return t > 0.0f ? t : CLR_INF_F;
        }
        if (r > 0.0f && fr == 0.0f) return r;
    }
    return CLR_INF_F;
}
__device__ __forceinline__ float f_surface_hit(float x, float y, float z, float vx, float vy, float vz, float zmean,
                                               float R, int model, float dh, float core) {
    if (model == 0 || dh <= 0.0f) {
        if (fabsf(vz) <= 1e-14f) return CLR_INF_F;
        const float t = (zmean - z) / vz;
        return (t > 0.0f) ? t : CLR_INF_F;
    }
    return f_surface_hit_curved(x, y, z, vx, vy, vz, zmean, R, model, dh, core);
}

/* unit normal into the water (:1768-1779) */
__device__ __forceinline__ void o_surface_normal(float x, float y, float R, int model, float dh, float core, float* nx, float* ny,
                                    float* nz) {
    if (model == 0 || dh <= 0.0f) { *nx = 0.0f; *ny = 0.0f; *nz = -1.0f; return; }
    if (model == 1) {
        float aa = dh / (R * R);
        *nx = 2.0f * aa * x; *ny = 2.0f * aa * y; *nz = -1.0f;
        o_normalize(nx, ny, nz);
        return;
    }
    if (model == 3) {  // dz/dr = 2 k r inside the core, 2 k a^4 / r^3 outside
        const RankineF g = f_rankine(0.0f, R, dh, core);
        const float q = x * x + y * y;
        const float fac = (q <= g.a2) ? 2.0f * g.k : 2.0f * g.k * g.a2 * g.a2 / (q * q);
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
__device__ __forceinline__ void o_perp_basis(float vx, float vy, float vz, float* e1x, float* e1y, float* e1z, float* e2x,
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

// Cell and weights of the bilinear lookup at (x, y, z): the same for every size bin, so a loop over
// bins computes them once (the arithmetic is the reference's, so the values are bit-identical).
struct o_grid_w {
    long long i, k;
    double tr, tz;
    int ok;
};
__device__ __forceinline__ o_grid_w o_grid_weights(const o_field* f, float x, float y, float z) {
    o_grid_w w;
    const int NR = f->grid_nr, NZ = f->grid_nz;
    w.ok = !(NR < 2 || NZ < 2 || !(f->grid_zmax > f->zmin));
    if (!w.ok) { w.i = w.k = 0; w.tr = w.tz = 0.0; return w; }
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
    w.i = i; w.k = k; w.tr = tr; w.tz = tz;
    return w;
}
__device__ __forceinline__ double o_grid_sample_w(const o_field* f, const o_grid_w& w, int pidx) {
    if (!w.ok) return 1.0;
    const long long NZ = f->grid_nz;
    const double* G = f->grid + (long long)pidx * ((long long)f->grid_nr * NZ) + w.i * NZ + w.k;
    double q00 = G[0], q10 = G[NZ], q01 = G[1], q11 = G[NZ + 1];
    double q0 = (1.0 - w.tr) * q00 + w.tr * q10, q1 = (1.0 - w.tr) * q01 + w.tr * q11;
    return fmax((1.0 - w.tz) * q0 + w.tz * q1, 0.0);
}
__device__ double o_grid_sample(const o_field* f, int pidx, float x, float y, float z) {
    const o_grid_w w = o_grid_weights(f, x, y, z);
    return o_grid_sample_w(f, w, pidx);
}
__device__ double o_local_scale(const o_field* f, int pidx, float x, float y, float z) {
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
template <class S>
__device__ int o_sample_local_bin(S* s, const o_field* f, const double* mu_bin, float x, float y, float z,
                              double local_total) {
    if (!(local_total > 0.0)) return 0;
    double target = (double)uniform(s) * local_total, cum = 0.0;
    if (f->model == 3) {
        const o_grid_w w = o_grid_weights(f, x, y, z);
        for (int i = 0; i < f->n_bins; ++i) {
            cum += mu_bin[i] * o_grid_sample_w(f, w, i);
            if (target <= cum) return i;
        }
        return f->n_bins > 0 ? f->n_bins - 1 : 0;
    }
    for (int i = 0; i < f->n_bins; ++i) {
        double sc = o_local_scale(f, i, x, y, z);
        cum += mu_bin[i] * sc;
        if (target <= cum) return i;
    }
    return f->n_bins > 0 ? f->n_bins - 1 : 0;
}

}  // namespace
}  // namespace clr
