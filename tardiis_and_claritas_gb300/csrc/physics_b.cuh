// Device physics, part B: Smith-Beckmann rough microsurface, particle
// interactions, Mie angle sampling, the connected acrylic solid, headspace and
// bottom disc. Same conventions as physics_a.cuh.
#pragma once
#include "physics_a.cuh"
#include "device_scene.cuh"

namespace clr {
namespace {  // header-only device code: internal linkage in every translation unit
/* microsurface outcomes and failure subcodes (:1800-1838) */
enum { OM_INTERSECTION = 1, OM_ESCAPE = 2, OM_NUMERICAL = 3, OM_WATCHDOG = 4 };
enum {
    OF_NONE = 0, OF_VNDF_PROJECTED_AREA = 10, OF_VNDF_CDF = 11, OF_VNDF_INVERSE_CDF = 12, OF_VNDF_VISIBILITY = 13,
    OF_VNDF_NORMALIZATION = 14, OF_HEIGHT_SAMPLE = 21, OF_HEIGHT_LAMBDA = 23, OF_HEIGHT_C0 = 24,
    OF_HEIGHT_LOG_C0 = 25, OF_HEIGHT_G1 = 26, OF_HEIGHT_ESCAPE_PROB = 27, OF_HEIGHT_RANDOM = 28,
    OF_HEIGHT_LOG_CNEXT = 29, OF_MICROFACET_NORMAL = 30, OF_REFLECTION_VECTOR = 31, OF_REFRACTION_VECTOR = 32,
    OF_SIDE_STATE = 33, OF_NONFINITE_DIRECTION = 34, OF_FRESNEL = 35, OF_HEIGHT_CNEXT_RANGE = 36,
    OF_HEIGHT_INVERSE_CDF = 37, OF_HEIGHT_OUTPUT = 38, OF_MICRO_WATCHDOG = 40
};
/* production failure codes and subcodes (:1844-1895) */
enum {
    OP_OK = 0, OP_MICRO_NUMERICAL = 1, OP_MICRO_WATCHDOG = 2, OP_MACRO_GEOMETRY = 3, OP_MACRO_BOUNCE_LIMIT = 4,
    OP_ACRYLIC_NO_INTERSECTION = 5, OP_ACRYLIC_BOUNCE_LIMIT = 6, OP_BOTTOM_GEOMETRY = 7,
    OP_WATER_NO_BOUNDARY = 9, OP_ITERATION_LIMIT = 10, OP_NONFINITE_POSITION = 11, OP_NONFINITE_DIRECTION = 12,
    OP_INVALID_MEDIUM = 13, OP_OTHER = 15, OP_SPHEROID_GEOMETRY = 16, OP_HEADSPACE_NO_BOUNDARY = 17,
    OP_MAJORANT_VIOLATION = 18
};
enum {
    OS_NONE = 0, OS_SPHERE_ENTRY_SIDE = 1001, OS_SPHERE_CHORD = 1002, OS_SPHERE_EXIT_SIDE = 1003,
    OS_SPHERE_INTERNAL_SIDE = 1004, OS_SPHERE_BOUNCE_LIMIT = 1005, OS_SPHEROID_ASPECT = 1101,
    OS_SPHEROID_AXES = 1102, OS_SPHEROID_ENTRY = 1103, OS_SPHEROID_CHORD = 1104, OS_SPHEROID_EXIT_SIDE = 1105,
    OS_SPHEROID_INTERNAL_SIDE = 1106, OS_SPHEROID_BOUNCE_LIMIT = 1107, OS_ACRYLIC_NO_INTERSECTION = 2001,
    OS_ACRYLIC_BOUNCE_LIMIT = 2002, OS_BOTTOM_TOPOLOGY = 2104, OS_WATER_NO_BOUNDARY = 3001,
    OS_ITERATION_LIMIT = 3002, OS_NONFINITE_POSITION = 3003, OS_NONFINITE_DIRECTION = 3004,
    OS_WATER_OUTSIDE = 3005, OS_HEADSPACE_NO_BOUNDARY = 3006, OS_MAJORANT = 4001
};

__device__ __forceinline__ double o_pos_inf(void) { return HUGE_VAL; }
__device__ __forceinline__ void o_setf(int* code, int v) { if (code) *code = v; }

/* B(x) = 1 - x sqrt(pi) erfcx(x) (:1925-1939) */
__device__ double o_tail_B(double x) {
    if (!(x >= 0.0) || !isfinite(x)) return -1.0;
    const double SQRT_PI = 1.77245385090551602729816748334114518;
    if (x < 5.0) {
        double e = exp(x * x) * erfc(x);
        double b = 1.0 - x * SQRT_PI * e;
        return (isfinite(b) && b > 0.0) ? b : -1.0;
    }
    double y = 1.0 / (x * x);
    double b = 0.5 * y - 0.75 * y * y + 1.875 * y * y * y - 6.5625 * y * y * y * y + 29.53125 * y * y * y * y * y -
               162.421875 * y * y * y * y * y * y + 1055.7421875 * y * y * y * y * y * y * y;
    return (isfinite(b) && b > 0.0) ? b : -1.0;
}
/* alpha=1 visible-slope marginal CDF, ordinary branch (:1944-1957) */
__device__ int o_visible_cdf(double slope, double slope_i, double* out) {
    if (!out || !isfinite(slope) || !isfinite(slope_i)) return 0;
    if (slope >= slope_i) { *out = 1.0; return 1; }
    const double K = 0.28209479177387814347403972578038629;
    double q = K * exp(-slope_i * slope_i) + 0.5 * slope_i * erfc(-slope_i);
    if (!(q > 0.0) || !isfinite(q)) return 0;
    double n = K * exp(-slope * slope) + 0.5 * slope_i * erfc(-slope);
    double f = n / q;
    if (!isfinite(f)) return 0;
    if (f < 0.0 && f > -1.0e-13) f = 0.0;
    if (f > 1.0 && f < 1.0 + 1.0e-13) f = 1.0;
    if (f < 0.0 || f > 1.0) return 0;
    *out = f;
    return 1;
}
/* signed-cot visible-slope sampler (:1965-2038) */
__device__ int o_sample11(double slope_i, double U1, double U2, double* slope_x, double* slope_y, int* fc) {
    o_setf(fc, OF_NONE);
    if (!slope_x || !slope_y || !isfinite(U1) || !isfinite(U2)) { o_setf(fc, OF_VNDF_CDF); return 0; }
    double u1 = U1, u2 = U2;
    if (!(u1 > 0.0 && u1 < 1.0) || !(u2 > 0.0 && u2 < 1.0)) { o_setf(fc, OF_VNDF_CDF); return 0; }
    const double COT_1E4 = 9999.999966666666;
    if (isinf(slope_i) || slope_i > COT_1E4) {
        if (slope_i < 0.0) { o_setf(fc, OF_VNDF_PROJECTED_AREA); return 0; }
        double r = sqrt(-log(u1)), phi = 2.0 * CLR_PI_D * u2;
        double sx = r * cos(phi), sy = r * sin(phi);
        if (!isfinite(sx) || !isfinite(sy)) { o_setf(fc, OF_VNDF_INVERSE_CDF); return 0; }
        *slope_x = sx; *slope_y = sy;
        return 1;
    }
    if (!isfinite(slope_i)) { o_setf(fc, OF_VNDF_PROJECTED_AREA); return 0; }
    double sx = 0.0;
    if (slope_i < -1.0) {
        double x = -slope_i, Bx = o_tail_B(x);
        if (!(Bx > 0.0) || !isfinite(Bx)) { o_setf(fc, OF_VNDF_PROJECTED_AREA); return 0; }
        double target = log(u1), lo = 0.0, hi = fmax(1.0 / x, 1.0e-12);
        int bracketed = 0;
        for (int it = 0; it < 64; ++it) {
            double y = x + hi, By = o_tail_B(y);
            if (!(By > 0.0) || !isfinite(By)) { o_setf(fc, OF_VNDF_CDF); return 0; }
            double Cc = hi / y + (x / y) * By;
            if (!(Cc > 0.0) || !isfinite(Cc)) { o_setf(fc, OF_VNDF_CDF); return 0; }
            double lr = -(2.0 * x * hi + hi * hi) + log(Cc / Bx);
            if (!isfinite(lr)) { o_setf(fc, OF_VNDF_CDF); return 0; }
            if (lr <= target) { bracketed = 1; break; }
            hi *= 2.0;
            if (!isfinite(hi)) { o_setf(fc, OF_VNDF_INVERSE_CDF); return 0; }
        }
        if (!bracketed) { o_setf(fc, OF_VNDF_INVERSE_CDF); return 0; }
        for (int it = 0; it < 52; ++it) {
            double mid = 0.5 * (lo + hi), y = x + mid, By = o_tail_B(y);
            if (!(By > 0.0) || !isfinite(By)) { o_setf(fc, OF_VNDF_CDF); return 0; }
            double Cc = mid / y + (x / y) * By;
            if (!(Cc > 0.0) || !isfinite(Cc)) { o_setf(fc, OF_VNDF_CDF); return 0; }
            double lr = -(2.0 * x * mid + mid * mid) + log(Cc / Bx);
            if (!isfinite(lr)) { o_setf(fc, OF_VNDF_CDF); return 0; }
            if (lr > target) lo = mid; else hi = mid;
        }
        sx = -(x + 0.5 * (lo + hi));
    } else {
        double lo = fmin(-1.0, slope_i - 1.0), hi = slope_i, flo = 1.0;
        int bracketed = 0;
        for (int it = 0; it < 64; ++it) {
            if (!o_visible_cdf(lo, slope_i, &flo)) { o_setf(fc, OF_VNDF_CDF); return 0; }
            if (flo <= u1) { bracketed = 1; break; }
            lo = (lo < 0.0) ? 2.0 * lo : lo - 1.0;
            if (!isfinite(lo)) { o_setf(fc, OF_VNDF_INVERSE_CDF); return 0; }
        }
        if (!bracketed) { o_setf(fc, OF_VNDF_INVERSE_CDF); return 0; }
        for (int it = 0; it < 48; ++it) {
            double mid = 0.5 * (lo + hi), fm = 0.0;
            if (!o_visible_cdf(mid, slope_i, &fm)) { o_setf(fc, OF_VNDF_CDF); return 0; }
            if (fm < u1) lo = mid; else hi = mid;
        }
        sx = 0.5 * (lo + hi);
    }
    double ey = 2.0 * u2 - 1.0;
    if (!(ey > -1.0 && ey < 1.0) || !isfinite(ey)) { o_setf(fc, OF_VNDF_INVERSE_CDF); return 0; }
    double sy = erfinv(ey);
    if (!isfinite(sx) || !isfinite(sy)) { o_setf(fc, OF_VNDF_INVERSE_CDF); return 0; }
    *slope_x = sx; *slope_y = sy;
    return 1;
}
/* signed Beckmann VNDF normal in the TOP-oriented frame (:2075-2132) */
template <class S>
__device__ int o_vndf_normal(S* s, float alpha, float bx, float by, float bz, float wx, float wy, float wz,
                         double* mx, double* my, double* mz, int* fc) {
    o_setf(fc, OF_NONE);
    if (!(alpha >= 0.0f) || !isfinite(alpha) || !s || !mx || !my || !mz) { o_setf(fc, OF_VNDF_NORMALIZATION); return 0; }
    o_normalize(&bx, &by, &bz);
    o_normalize(&wx, &wy, &wz);
    if (!isfinite(bx) || !isfinite(by) || !isfinite(bz) || !isfinite(wx) || !isfinite(wy) || !isfinite(wz)) {
        o_setf(fc, OF_NONFINITE_DIRECTION); return 0;
    }
    if (alpha <= 1.0e-8f) {
        double vd = (double)wx * bx + (double)wy * by + (double)wz * bz;
        if (!(vd > 0.0)) { o_setf(fc, OF_VNDF_VISIBILITY); return 0; }
        *mx = (double)bx; *my = (double)by; *mz = (double)bz;
        return 1;
    }
    float t1x, t1y, t1z, t2x, t2y, t2z;
    o_perp_basis(bx, by, bz, &t1x, &t1y, &t1z, &t2x, &t2y, &t2z);
    double lx = (double)wx * t1x + (double)wy * t1y + (double)wz * t1z;
    double ly = (double)wx * t2x + (double)wy * t2y + (double)wz * t2z;
    double lz = (double)wx * bx + (double)wy * by + (double)wz * bz;
    double sxv = (double)alpha * lx, syv = (double)alpha * ly, szv = lz;
    double vl = sqrt(sxv * sxv + syv * syv + szv * szv);
    if (!(vl > 0.0) || !isfinite(vl)) { o_setf(fc, OF_VNDF_NORMALIZATION); return 0; }
    sxv /= vl; syv /= vl; szv /= vl;
    double radial = hypot(sxv, syv), slope_i = 0.0;
    if (radial == 0.0) {
        if (szv > 0.0) slope_i = o_pos_inf();
        else { o_setf(fc, OF_VNDF_PROJECTED_AREA); return 0; }
    } else {
        slope_i = szv / radial;
        if (!isfinite(slope_i)) { o_setf(fc, OF_VNDF_PROJECTED_AREA); return 0; }
    }
    double sx0 = 0.0, sy0 = 0.0;
    int f2 = OF_NONE;
    double U1 = open_uniform(s), U2 = open_uniform(s);
    if (!o_sample11(slope_i, U1, U2, &sx0, &sy0, &f2)) { o_setf(fc, f2 ? f2 : OF_VNDF_INVERSE_CDF); return 0; }
    double phi = atan2(syv, sxv), cp = cos(phi), sp = sin(phi);
    double tx = cp * sx0 - sp * sy0, ty = sp * sx0 + cp * sy0;
    double sx = (double)alpha * tx, sy = (double)alpha * ty;
    if (!isfinite(sx) || !isfinite(sy)) { o_setf(fc, OF_MICROFACET_NORMAL); return 0; }
    double invn = 1.0 / sqrt(sx * sx + sy * sy + 1.0);
    if (!(invn > 0.0) || !isfinite(invn)) { o_setf(fc, OF_VNDF_NORMALIZATION); return 0; }
    double nlx = -sx * invn, nly = -sy * invn, nlz = invn;
    double nx = nlx * t1x + nly * t2x + nlz * bx;
    double ny = nlx * t1y + nly * t2y + nlz * by;
    double nz = nlx * t1z + nly * t2z + nlz * bz;
    double nn = sqrt(nx * nx + ny * ny + nz * nz);
    if (!(nn > 0.0) || !isfinite(nn)) { o_setf(fc, OF_VNDF_NORMALIZATION); return 0; }
    nx /= nn; ny /= nn; nz /= nn;
    double top = nx * bx + ny * by + nz * bz;
    double vis = nx * wx + ny * wy + nz * wz;
    if (!(top > 0.0)) { o_setf(fc, OF_MICROFACET_NORMAL); return 0; }
    if (!(vis > 0.0)) { o_setf(fc, OF_VNDF_VISIBILITY); return 0; }
    *mx = nx; *my = ny; *mz = nz;
    return 1;
}
/* Smith Lambda over the full sphere (:2170-2188) */
__device__ double o_smith_lambda(float wx, float wy, float wz, float bx, float by, float bz, float alpha) {
    double c = (double)wx * bx + (double)wy * by + (double)wz * bz;
    if (!isfinite(c) || !isfinite(alpha) || !(alpha >= 0.0f)) return __longlong_as_double(0x7ff8000000000000LL);
    c = fmax(-1.0, fmin(1.0, c));
    double ss2 = fmax(0.0, 1.0 - c * c);
    if (ss2 == 0.0) return c >= 0.0 ? 0.0 : -1.0;
    if (c == 0.0) return copysign(o_pos_inf(), c);
    if (alpha == 0.0f) return c >= 0.0 ? 0.0 : -1.0;
    double aa = fabs(c) / ((double)alpha * sqrt(ss2));
    if (!(aa > 0.0) || !isfinite(aa)) return c >= 0.0 ? 0.0 : -1.0;
    const double SQRT_PI = 1.77245385090551602729816748334114518;
    double B = o_tail_B(aa);
    if (!(B > 0.0) || !isfinite(B)) return __longlong_as_double(0x7ff8000000000000LL);
    double logpref = -(aa * aa) - log(2.0 * SQRT_PI * aa);
    double lp = exp(logpref) * B;
    if (!(lp >= 0.0) || !isfinite(lp)) return __longlong_as_double(0x7ff8000000000000LL);
    return c >= 0.0 ? lp : (-1.0 - lp);
}
__device__ __forceinline__ double o_C1(double h) { return fmin(1.0, fmax(0.0, 0.5 * (h + 1.0))); }
__device__ __forceinline__ double o_invC1(double u) { return 2.0 * fmin(1.0, fmax(0.0, u)) - 1.0; }
/* stable Smith height sampler (:2217-2300) */
__device__ int o_height_u(double U, float wx, float wy, float wz, float bx, float by, float bz, float alpha, float h,
                      float* out_h, int* fc) {
    o_setf(fc, OF_NONE);
    if (!out_h || !isfinite(U) || !isfinite(wx) || !isfinite(wy) || !isfinite(wz) || !isfinite(h) ||
        !(alpha >= 0.0f) || !isfinite(alpha)) { o_setf(fc, OF_HEIGHT_RANDOM); return OM_NUMERICAL; }
    if (!(U > 0.0 && U < 1.0)) { o_setf(fc, OF_HEIGHT_RANDOM); return OM_NUMERICAL; }
    double c = (double)wx * bx + (double)wy * by + (double)wz * bz;
    if (!isfinite(c)) { o_setf(fc, OF_NONFINITE_DIRECTION); return OM_NUMERICAL; }
    c = fmax(-1.0, fmin(1.0, c));
    double C0 = o_C1((double)h);
    if (!(C0 >= 0.0 && C0 <= 1.0) || !isfinite(C0)) { o_setf(fc, OF_HEIGHT_C0); return OM_NUMERICAL; }
    double ss2 = fmax(0.0, 1.0 - c * c);
    if (ss2 == 0.0) {
        if (c > 0.0) return OM_ESCAPE;
        if (c < 0.0) {
            double Cnext = U * C0, hn = o_invC1(Cnext);
            if (!isfinite(hn)) { o_setf(fc, OF_HEIGHT_INVERSE_CDF); return OM_NUMERICAL; }
            *out_h = (float)hn;
            return OM_INTERSECTION;
        }
        *out_h = h;
        return OM_INTERSECTION;
    }
    if (c == 0.0) { *out_h = h; return OM_INTERSECTION; }
    double lam = o_smith_lambda(wx, wy, wz, bx, by, bz, alpha);
    if (isnan(lam)) { o_setf(fc, OF_HEIGHT_LAMBDA); return OM_NUMERICAL; }
    if (c > 0.0) {
        if (!(lam >= 0.0)) { o_setf(fc, OF_HEIGHT_LAMBDA); return OM_NUMERICAL; }
        if (C0 <= 0.0) return OM_ESCAPE;
        if (C0 >= 1.0) return OM_ESCAPE;
        if (lam == 0.0) return OM_ESCAPE;
        double logC0 = log(C0);
        if (!isfinite(logC0)) { o_setf(fc, OF_HEIGHT_LOG_C0); return OM_NUMERICAL; }
        double logG1 = lam * logC0;
        if (!(logG1 <= 0.0) || !isfinite(logG1)) { o_setf(fc, OF_HEIGHT_G1); return OM_NUMERICAL; }
        double p_int = -expm1(logG1);
        if (!(p_int >= 0.0 && p_int <= 1.0) || !isfinite(p_int)) { o_setf(fc, OF_HEIGHT_ESCAPE_PROB); return OM_NUMERICAL; }
        if (U > p_int) return OM_ESCAPE;
        double log1mU = log1p(-U);
        if (!isfinite(log1mU)) { o_setf(fc, OF_HEIGHT_RANDOM); return OM_NUMERICAL; }
        double logCnext = logC0 - log1mU / lam;
        if (!isfinite(logCnext)) { o_setf(fc, OF_HEIGHT_LOG_CNEXT); return OM_NUMERICAL; }
        const double BOUND_TOL = 64.0 * 2.2204460492503130808472633361816e-16;
        if (logCnext > BOUND_TOL) { o_setf(fc, OF_HEIGHT_CNEXT_RANGE); return OM_NUMERICAL; }
        if (logCnext > 0.0) logCnext = 0.0;
        double Cnext = exp(logCnext);
        if (!(Cnext >= 0.0 && Cnext <= 1.0) || !isfinite(Cnext)) { o_setf(fc, OF_HEIGHT_CNEXT_RANGE); return OM_NUMERICAL; }
        double hn = o_invC1(Cnext);
        if (!isfinite(hn)) { o_setf(fc, OF_HEIGHT_INVERSE_CDF); return OM_NUMERICAL; }
        *out_h = (float)hn;
        if (!isfinite(*out_h)) { o_setf(fc, OF_HEIGHT_OUTPUT); return OM_NUMERICAL; }
        return OM_INTERSECTION;
    }
    if (!(lam <= -1.0) || !isfinite(lam)) { o_setf(fc, OF_HEIGHT_LAMBDA); return OM_NUMERICAL; }
    if (C0 <= 0.0) { *out_h = -1.0f; return OM_INTERSECTION; }
    double logC0 = log(C0);
    if (!isfinite(logC0)) { o_setf(fc, OF_HEIGHT_LOG_C0); return OM_NUMERICAL; }
    double log1mU = log1p(-U);
    if (!isfinite(log1mU)) { o_setf(fc, OF_HEIGHT_RANDOM); return OM_NUMERICAL; }
    double logCnext = logC0 - log1mU / lam;
    if (!isfinite(logCnext)) { o_setf(fc, OF_HEIGHT_LOG_CNEXT); return OM_NUMERICAL; }
    if (logCnext > 0.0) { o_setf(fc, OF_HEIGHT_CNEXT_RANGE); return OM_NUMERICAL; }
    double Cnext = exp(logCnext);
    if (!(Cnext >= 0.0 && Cnext <= C0 * (1.0 + 8.0e-15)) || !isfinite(Cnext)) { o_setf(fc, OF_HEIGHT_CNEXT_RANGE); return OM_NUMERICAL; }
    double hn = o_invC1(Cnext);
    if (!isfinite(hn)) { o_setf(fc, OF_HEIGHT_INVERSE_CDF); return OM_NUMERICAL; }
    *out_h = (float)hn;
    if (!isfinite(*out_h)) { o_setf(fc, OF_HEIGHT_OUTPUT); return OM_NUMERICAL; }
    return OM_INTERSECTION;
}
template <class S>
__device__ int o_height(S* s, float wx, float wy, float wz, float bx, float by, float bz, float alpha, float h,
                    float* out_h, int* fc) {
    double U = open_uniform(s);
    if (!(U > 0.0 && U < 1.0) || !isfinite(U)) { o_setf(fc, OF_HEIGHT_RANDOM); return OM_NUMERICAL; }
    return o_height_u(U, wx, wy, wz, bx, by, bz, alpha, h, out_h, fc);
}
/* rough branch of the microsurface walk, kept out of line: it is the FP64-heavy rare path */
template <class S>
__device__ __noinline__ int o_micro_walk_rough(S* s, float alpha, int watchdog, float bx, float by, float bz, float n_top,
                                               float k_top, float n_bottom, float k_bottom, float* dx, float* dy,
                                               float* dz, int* out_top, int* scatter_order, int* fc) {
    float h = 1.0f + (2.0f * fminf(fmaxf(0.999f, 0.0f), 1.0f) - 1.0f);
    int outside = 1, order = 0;
    for (int it = 0; it < watchdog; ++it) {
        float nh = 0.0f;
        int hs, f2 = OF_NONE;
        if (outside) {
            hs = o_height(s, *dx, *dy, *dz, bx, by, bz, alpha, h, &nh, &f2);
            if (hs == OM_ESCAPE) { *out_top = 1; *scatter_order = order; return OM_ESCAPE; }
        } else {
            float tmp = 0.0f;
            hs = o_height(s, -(*dx), -(*dy), -(*dz), bx, by, bz, alpha, -h, &tmp, &f2);
            if (hs == OM_ESCAPE) { *out_top = 0; *scatter_order = order; return OM_ESCAPE; }
            if (hs == OM_INTERSECTION) nh = -tmp;
        }
        if (hs != OM_INTERSECTION || !isfinite(nh)) {
            *scatter_order = order; o_setf(fc, f2 ? f2 : OF_HEIGHT_SAMPLE); return OM_NUMERICAL;
        }
        h = nh;
        ++order;
        float wix = -(*dx), wiy = -(*dy), wiz = -(*dz);
        double mx, my, mz;
        f2 = OF_NONE;
        if (outside) {
            if (!o_vndf_normal(s, alpha, bx, by, bz, wix, wiy, wiz, &mx, &my, &mz, &f2)) {
                *scatter_order = order; o_setf(fc, f2 ? f2 : OF_VNDF_INVERSE_CDF); return OM_NUMERICAL;
            }
        } else {
            double tx, ty, tz;
            if (!o_vndf_normal(s, alpha, bx, by, bz, -wix, -wiy, -wiz, &tx, &ty, &tz, &f2)) {
                *scatter_order = order; o_setf(fc, f2 ? f2 : OF_VNDF_INVERSE_CDF); return OM_NUMERICAL;
            }
            mx = -tx; my = -ty; mz = -tz;
        }
        double vis = (double)wix * mx + (double)wiy * my + (double)wiz * mz;
        if (!isfinite(mx) || !isfinite(my) || !isfinite(mz)) { *scatter_order = order; o_setf(fc, OF_MICROFACET_NORMAL); return OM_NUMERICAL; }
        if (!(vis > 0.0)) { *scatter_order = order; o_setf(fc, OF_VNDF_VISIBILITY); return OM_NUMERICAL; }
        double ci_d = fmin(1.0, fmax(0.0, vis));
        float ci = (float)ci_d;
        float n1 = outside ? n_top : n_bottom, k1 = outside ? k_top : k_bottom;
        float n2 = outside ? n_bottom : n_top, k2 = outside ? k_bottom : k_top;
        if (!(n1 > 0.0f && n2 > 0.0f)) { o_setf(fc, OF_REFRACTION_VECTOR); return OM_NUMERICAL; }
        float R, ts, tn;
        if (!o_particle_interface(ci, n1, k1, n2, k2, &R, &ts, &tn)) { o_setf(fc, OF_FRESNEL); return OM_NUMERICAL; }
        if (!isfinite(R)) { o_setf(fc, OF_FRESNEL); return OM_NUMERICAL; }
        double ox_d, oy_d, oz_d;
        if (uniform(s) < R) {
            double dd = (double)(*dx) * mx + (double)(*dy) * my + (double)(*dz) * mz;
            ox_d = (double)(*dx) - 2.0 * dd * mx; oy_d = (double)(*dy) - 2.0 * dd * my; oz_d = (double)(*dz) - 2.0 * dd * mz;
        } else {
            float tx, ty, tz;
            if (!o_particle_refract(*dx, *dy, *dz, (float)mx, (float)my, (float)mz, n1, k1, n2, k2, &tx, &ty, &tz)) {
                o_setf(fc, OF_REFRACTION_VECTOR); return OM_NUMERICAL;
            }
            ox_d = tx; oy_d = ty; oz_d = tz;
            outside = 1 - outside;
        }
        double qn = sqrt(ox_d * ox_d + oy_d * oy_d + oz_d * oz_d);
        if (!(qn > 0.0) || !isfinite(qn) || !isfinite(ox_d) || !isfinite(oy_d) || !isfinite(oz_d)) {
            *scatter_order = order; o_setf(fc, OF_REFRACTION_VECTOR); return OM_NUMERICAL;
        }
        ox_d /= qn; oy_d /= qn; oz_d /= qn;
        float ox = (float)ox_d, oy = (float)oy_d, oz = (float)oz_d;
        if (!isfinite(ox) || !isfinite(oy) || !isfinite(oz)) { *scatter_order = order; o_setf(fc, OF_NONFINITE_DIRECTION); return OM_NUMERICAL; }
        o_normalize(&ox, &oy, &oz);
        if (!isfinite(ox) || !isfinite(oy) || !isfinite(oz)) { *scatter_order = order; o_setf(fc, OF_NONFINITE_DIRECTION); return OM_NUMERICAL; }
        *dx = ox; *dy = oy; *dz = oz;
    }
    *scatter_order = order;
    o_setf(fc, OF_MICRO_WATCHDOG);
    return OM_WATCHDOG;
}

/* rough dielectric microsurface random walk (:2323-2422) */
template <class S>
__device__ __forceinline__ int o_micro_walk(S* s, float alpha, int watchdog, float bx, float by, float bz, float n_top,
                        float k_top, float n_bottom, float k_bottom, float* dx, float* dy, float* dz, int* out_top,
                        int* scatter_order, int* fc) {
    o_setf(fc, OF_NONE);
    o_normalize(&bx, &by, &bz);
    o_normalize(dx, dy, dz);
    *scatter_order = 0;
    if (!isfinite(bx) || !isfinite(by) || !isfinite(bz) || !isfinite(*dx) || !isfinite(*dy) || !isfinite(*dz)) {
        o_setf(fc, OF_NONFINITE_DIRECTION); return OM_NUMERICAL;
    }
    if (o_dot(*dx, *dy, *dz, bx, by, bz) >= -1.0e-7f) { o_setf(fc, OF_SIDE_STATE); return OM_NUMERICAL; }
    if (watchdog < 1) { o_setf(fc, OF_MICRO_WATCHDOG); return OM_WATCHDOG; }
    if (alpha <= 1.0e-7f) {
        float wi_x = -(*dx), wi_y = -(*dy), wi_z = -(*dz);
        float ci = fminf(fmaxf(o_dot(wi_x, wi_y, wi_z, bx, by, bz), 0.0f), 1.0f);
        float R, ts, tn;
        if (!o_particle_interface(ci, n_top, k_top, n_bottom, k_bottom, &R, &ts, &tn)) { o_setf(fc, OF_FRESNEL); return OM_NUMERICAL; }
        if (!isfinite(R)) { o_setf(fc, OF_FRESNEL); return OM_NUMERICAL; }
        float ox, oy, oz;
        if (uniform(s) < R) {
            o_reflect(*dx, *dy, *dz, bx, by, bz, &ox, &oy, &oz);
            *out_top = 1;
            if (!isfinite(ox) || !isfinite(oy) || !isfinite(oz)) { o_setf(fc, OF_REFLECTION_VECTOR); return OM_NUMERICAL; }
        } else {
            if (!o_particle_refract(*dx, *dy, *dz, bx, by, bz, n_top, k_top, n_bottom, k_bottom, &ox, &oy, &oz)) {
                o_setf(fc, OF_REFRACTION_VECTOR); return OM_NUMERICAL;
            }
            *out_top = 0;
        }
        if (!isfinite(ox) || !isfinite(oy) || !isfinite(oz)) { o_setf(fc, OF_NONFINITE_DIRECTION); return OM_NUMERICAL; }
        *dx = ox; *dy = oy; *dz = oz;
        *scatter_order = 1;
        return OM_ESCAPE;
    }
    return o_micro_walk_rough(s, alpha, watchdog, bx, by, bz, n_top, k_top, n_bottom, k_bottom, dx, dy, dz, out_top,
                              scatter_order, fc);
}

/* ---------------- particle geometry and interaction (:2436-2622) ---------------- */
template <class S>
__device__ void o_sphere_geometry(S* s, float radius, float x, float y, float z, float vx, float vy, float vz,
                              float* rho_o, float* phi_o, float* gx, float* gy, float* gz) {
    (void)radius; (void)x; (void)y; (void)z;
    float rho = sqrtf(fminf(fmaxf(uniform(s), 0.0f), 0.99999994f));
    float ci = sqrtf(fmaxf(0.0f, 1.0f - rho * rho));
    float phi = uniform(s) * 2.0f * CLR_PI_F;
    float e1x, e1y, e1z, e2x, e2y, e2z;
    o_perp_basis(vx, vy, vz, &e1x, &e1y, &e1z, &e2x, &e2y, &e2z);
    float qx = cosf(phi) * e1x + sinf(phi) * e2x;
    float qy = cosf(phi) * e1y + sinf(phi) * e2y;
    float qz = cosf(phi) * e1z + sinf(phi) * e2z;
    float gnx = -ci * vx + rho * qx, gny = -ci * vy + rho * qy, gnz = -ci * vz + rho * qz;
    o_normalize(&gnx, &gny, &gnz);
    *rho_o = rho; *phi_o = phi; *gx = gnx; *gy = gny; *gz = gnz;
}
/* finite sphere fits inside the water at its sampled centre (:2459-2495) */
__device__ int o_sphere_accessible(double cx, double cy, double cz, double radius, float Rin, float Zmin, float Zmean,
                               int model, float dh, float core) {
    double rc = hypot(cx, cy), rr = radius;
    double cclear = (double)Rin - rc;
    double wall = cclear - rr;
    double bottom = cz - rr - (double)Zmin;
    double rmin = fmax(0.0, rc - rr);
    double zsurf = (double)Zmean;
    if (model != 0 && dh > 0.0f) {
        double R = (double)Rin, d = (double)dh, a = (double)core;
        double q = rmin * rmin, R2 = R * R;
        if (model == 1) {
            zsurf = (double)Zmean + d * (q / R2 - 0.5);
        } else if (model == 3) {
            zsurf = d_rankine_z(d_rankine((double)Zmean, R, d, a), q);
        } else {
            double a2 = a * a;
            double H = d * (a2 + R2) / R2;
            double hbar = H * (1.0 - (a2 / R2) * log1p(R2 / a2));
            zsurf = (double)Zmean - hbar + H * q / (a2 + q);
        }
    }
    double top = zsurf - (cz + rr);
    double scale = fmax(fmax(fabs((double)Rin), fabs(cz)), fmax(rr, 1.0e-6));
    double tol = 128.0 * CLR_DBL_EPS * scale;
    return (wall >= -tol && bottom >= -tol && top >= -tol) ? 1 : 0;
}
typedef struct {
    int reflections, entry_reflections, internal_reflections, absorptions;
} o_pcount;

/* sphere entry -> chords -> exit with microsurface walks; 1 scattered, 2 absorbed, 0 failure (:2497-2599) */
template <class S>
__device__ int o_sphere_sampled(S* s, float n_medium, float n_particle, float k_particle, float wavelength,
                            float rough_alpha, float radius, int max_bounces, float gnx, float gny, float gnz,
                            double cx, double cy, double cz, float* x, float* y, float* z, float* vx, float* vy,
                            float* vz, float* internal_path, o_pcount* pc, int* pf, int* pfs, int* macro,
                            int* micro, float* wmul = nullptr) {
    *pf = OP_OK; *pfs = OS_NONE; *macro = 0; *micro = 0;
    if (radius <= 0.0f) return 1;
    const int WD = 4096;
    int top = 1, order = 0, mfc = OF_NONE;
    int ms = o_micro_walk(s, rough_alpha, WD, gnx, gny, gnz, n_medium, 0.0f, n_particle, k_particle, vx, vy, vz, &top,
                          &order, &mfc);
    *micro = order;
    if (ms != OM_ESCAPE) { *pf = (ms == OM_WATCHDOG) ? OP_MICRO_WATCHDOG : OP_MICRO_NUMERICAL; *pfs = mfc; return 0; }
    if (top) { pc->reflections++; pc->entry_reflections++; return 1; }
    if (o_dot(*vx, *vy, *vz, gnx, gny, gnz) >= 0.0f) { *pf = OP_MACRO_GEOMETRY; *pfs = OS_SPHERE_ENTRY_SIDE; return 0; }
    const double rr = (double)radius, rr2 = rr * rr;
    double qx = rr * (double)gnx, qy = rr * (double)gny, qz = rr * (double)gnz;
    double qn0 = sqrt(qx * qx + qy * qy + qz * qz);
    if (!(qn0 > 0.0) || !isfinite(qn0)) { *pf = OP_MACRO_GEOMETRY; *pfs = OS_SPHERE_CHORD; return 0; }
    qx *= rr / qn0; qy *= rr / qn0; qz *= rr / qn0;
    float alpha_abs = (wavelength > 0.0f && k_particle > 0.0f) ? (4.0f * CLR_PI_F * k_particle / wavelength) : 0.0f;
    for (int bounce = 0; bounce <= max_bounces; ++bounce) {
        *macro = bounce;
        double dvx = (double)(*vx), dvy = (double)(*vy), dvz = (double)(*vz);
        double A = dvx * dvx + dvy * dvy + dvz * dvz;
        double q2 = qx * qx + qy * qy + qz * qz;
        if (!(A > 0.0) || !isfinite(A) || !isfinite(q2)) { *pf = OP_MACRO_GEOMETRY; *pfs = OS_SPHERE_CHORD; return 0; }
        double qnorm = sqrt(q2);
        if (!(qnorm > 0.0) || !isfinite(qnorm)) { *pf = OP_MACRO_GEOMETRY; *pfs = OS_SPHERE_CHORD; return 0; }
        double qproj = rr / qnorm;
        qx *= qproj; qy *= qproj; qz *= qproj;
        double B = qx * dvx + qy * dvy + qz * dvz;
        if (!(B < 0.0) || !isfinite(B)) { *pf = OP_MACRO_GEOMETRY; *pfs = OS_SPHERE_INTERNAL_SIDE; return 0; }
        double chord = -2.0 * B / A;
        if (!(chord > 0.0) || !isfinite(chord)) { *pf = OP_MACRO_GEOMETRY; *pfs = OS_SPHERE_CHORD; return 0; }
        double tqx = qx + chord * dvx, tqy = qy + chord * dvy, tqz = qz + chord * dvz;
        double arrival = tqx * dvx + tqy * dvy + tqz * dvz;
        double tq2 = tqx * tqx + tqy * tqy + tqz * tqz;
        double err = fabs(tq2 - rr2);
        double tol = 512.0 * CLR_DBL_EPS * fmax(rr2, 1.0e-30);
        if (!(arrival > 0.0) || !isfinite(arrival) || !isfinite(tq2) || err > tol) {
            *pf = OP_MACRO_GEOMETRY; *pfs = OS_SPHERE_CHORD; return 0;
        }
        float chord_f = (float)chord;
        if (alpha_abs > 0.0f && wmul) {
            *wmul *= expf(-alpha_abs * chord_f);  // implicit capture: the chord's survival probability
        } else if (alpha_abs > 0.0f) {
            double dist = -log(open_uniform(s)) / (double)alpha_abs;
            if (dist < chord) {
                qx += dist * dvx; qy += dist * dvy; qz += dist * dvz;
                *x = (float)(cx + qx); *y = (float)(cy + qy); *z = (float)(cz + qz);
                *internal_path += (float)dist;
                pc->absorptions++;
                return 2;
            }
        }
        qx = tqx; qy = tqy; qz = tqz;
        *internal_path += chord_f;
        double qn = sqrt(qx * qx + qy * qy + qz * qz);
        if (!(qn > 0.0) || !isfinite(qn)) { *pf = OP_MACRO_GEOMETRY; *pfs = OS_SPHERE_CHORD; return 0; }
        double proj = rr / qn;
        qx *= proj; qy *= proj; qz *= proj;
        *x = (float)(cx + qx); *y = (float)(cy + qy); *z = (float)(cz + qz);
        float nox = (float)(qx / rr), noy = (float)(qy / rr), noz = (float)(qz / rr);
        o_normalize(&nox, &noy, &noz);
        float bx = -nox, by = -noy, bz = -noz;
        top = 1; order = 0; mfc = OF_NONE;
        ms = o_micro_walk(s, rough_alpha, WD, bx, by, bz, n_particle, k_particle, n_medium, 0.0f, vx, vy, vz, &top,
                          &order, &mfc);
        *micro = order;
        if (ms != OM_ESCAPE) { *pf = (ms == OM_WATCHDOG) ? OP_MICRO_WATCHDOG : OP_MICRO_NUMERICAL; *pfs = mfc; return 0; }
        if (!top) {
            if (o_dot(*vx, *vy, *vz, nox, noy, noz) <= 0.0f) { *pf = OP_MACRO_GEOMETRY; *pfs = OS_SPHERE_EXIT_SIDE; return 0; }
            return 1;
        }
        if (o_dot(*vx, *vy, *vz, nox, noy, noz) >= 0.0f) { *pf = OP_MACRO_GEOMETRY; *pfs = OS_SPHERE_INTERNAL_SIDE; return 0; }
        pc->reflections++;
        pc->internal_reflections++;
        if (bounce == max_bounces) { *pf = OP_MACRO_BOUNCE_LIMIT; *pfs = OS_SPHERE_BOUNCE_LIMIT; return 0; }
    }
    *pf = OP_OTHER; *pfs = OS_NONE;
    return 0;
}
/* FP32 versions of the sphere accessibility test and chord walk for the counter-based stream: the
 * same tests in the same order; the chord tolerance is scaled from DBL_EPS to FLT_EPS (chords are
 * relative to the sphere centre, so their relative accuracy is FP32's whatever the cell size) and
 * the accessibility test asks for a clearance of a few FP32 ulps instead of allowing an overlap. */
__device__ __forceinline__ int f_sphere_accessible(float cx, float cy, float cz, float radius, float Rin, float Zmin,
                                                   float Zmean, int model, float dh, float core) {
    const float rc = hypotf(cx, cy), rr = radius;
    const float wall = (Rin - rc) - rr;
    const float bottom = cz - rr - Zmin;
    const float rmin = fmaxf(0.0f, rc - rr);
    float zsurf = Zmean;
    if (model != 0 && dh > 0.0f) {
        const float q = rmin * rmin, R2 = Rin * Rin;
        if (model == 1) {
            zsurf = Zmean + dh * (q / R2 - 0.5f);
        } else if (model == 3) {
            zsurf = f_rankine_z(f_rankine(Zmean, Rin, dh, core), q);
        } else {
            const float a2 = core * core;
            const float H = dh * (a2 + R2) / R2;
            const float hbar = H * (1.0f - (a2 / R2) * log1pf(R2 / a2));
            zsurf = Zmean - hbar + H * q / (a2 + q);
        }
    }
    const float top = zsurf - (cz + rr);
    // The FP64 test accepts spheres within ~1e-15 m of the boundary. In FP32 the clearances carry
    // errors of a few ulps of the cell coordinates, so a sphere must clear every boundary by four of
    // them: a borderline sphere is rejected rather than allowed to intrude, and exit points on it
    // stay inside the water.
    const float scale = fmaxf(fmaxf(fabsf(Rin), fabsf(cz)), fmaxf(rr, 1.0e-6f));
    const float tol = 4.0f * 1.1920928955078125e-7f * scale;
    return (wall >= tol && bottom >= tol && top >= tol) ? 1 : 0;
}
template <class S>
__device__ int f_sphere_sampled(S* s, float n_medium, float n_particle, float k_particle, float wavelength,
                                float rough_alpha, float radius, int max_bounces, float gnx, float gny, float gnz,
                                float cx, float cy, float cz, float* x, float* y, float* z, float* vx, float* vy,
                                float* vz, float* internal_path, o_pcount* pc, int* pf, int* pfs, int* macro,
                                int* micro, float* wmul = nullptr) {
    const float FEPS = 1.1920928955078125e-7f;
    *pf = OP_OK; *pfs = OS_NONE; *macro = 0; *micro = 0;
    if (radius <= 0.0f) return 1;
    const int WD = 4096;
    int top = 1, order = 0, mfc = OF_NONE;
    int ms = o_micro_walk(s, rough_alpha, WD, gnx, gny, gnz, n_medium, 0.0f, n_particle, k_particle, vx, vy, vz, &top,
                          &order, &mfc);
    *micro = order;
    if (ms != OM_ESCAPE) { *pf = (ms == OM_WATCHDOG) ? OP_MICRO_WATCHDOG : OP_MICRO_NUMERICAL; *pfs = mfc; return 0; }
    if (top) { pc->reflections++; pc->entry_reflections++; return 1; }
    if (o_dot(*vx, *vy, *vz, gnx, gny, gnz) >= 0.0f) { *pf = OP_MACRO_GEOMETRY; *pfs = OS_SPHERE_ENTRY_SIDE; return 0; }
    const float rr = radius, rr2 = rr * rr;
    float qx = rr * gnx, qy = rr * gny, qz = rr * gnz;
    const float qn0 = sqrtf(qx * qx + qy * qy + qz * qz);
    if (!(qn0 > 0.0f) || !isfinite(qn0)) { *pf = OP_MACRO_GEOMETRY; *pfs = OS_SPHERE_CHORD; return 0; }
    qx *= rr / qn0; qy *= rr / qn0; qz *= rr / qn0;
    const float alpha_abs = (wavelength > 0.0f && k_particle > 0.0f) ? (4.0f * CLR_PI_F * k_particle / wavelength) : 0.0f;
    for (int bounce = 0; bounce <= max_bounces; ++bounce) {
        *macro = bounce;
        const float dvx = *vx, dvy = *vy, dvz = *vz;
        const float A = dvx * dvx + dvy * dvy + dvz * dvz;
        const float q2 = qx * qx + qy * qy + qz * qz;
        if (!(A > 0.0f) || !isfinite(A) || !isfinite(q2)) { *pf = OP_MACRO_GEOMETRY; *pfs = OS_SPHERE_CHORD; return 0; }
        const float qnorm = sqrtf(q2);
        if (!(qnorm > 0.0f) || !isfinite(qnorm)) { *pf = OP_MACRO_GEOMETRY; *pfs = OS_SPHERE_CHORD; return 0; }
        const float qproj = rr / qnorm;
        qx *= qproj; qy *= qproj; qz *= qproj;
        const float B = qx * dvx + qy * dvy + qz * dvz;
        if (!(B < 0.0f) || !isfinite(B)) { *pf = OP_MACRO_GEOMETRY; *pfs = OS_SPHERE_INTERNAL_SIDE; return 0; }
        const float chord = -2.0f * B / A;
        if (!(chord > 0.0f) || !isfinite(chord)) { *pf = OP_MACRO_GEOMETRY; *pfs = OS_SPHERE_CHORD; return 0; }
        const float tqx = qx + chord * dvx, tqy = qy + chord * dvy, tqz = qz + chord * dvz;
        const float arrival = tqx * dvx + tqy * dvy + tqz * dvz;
        const float tq2 = tqx * tqx + tqy * tqy + tqz * tqz;
        const float err = fabsf(tq2 - rr2);
        const float tol = 512.0f * FEPS * fmaxf(rr2, 1.0e-30f);
        if (!(arrival > 0.0f) || !isfinite(arrival) || !isfinite(tq2) || err > tol) {
            *pf = OP_MACRO_GEOMETRY; *pfs = OS_SPHERE_CHORD; return 0;
        }
        if (alpha_abs > 0.0f && wmul) {
            *wmul *= expf(-alpha_abs * chord);  // implicit capture: the chord's survival probability
        } else if (alpha_abs > 0.0f) {
            const float dist = -logf((float)open_uniform(s)) / alpha_abs;
            if (dist < chord) {
                qx += dist * dvx; qy += dist * dvy; qz += dist * dvz;
                *x = cx + qx; *y = cy + qy; *z = cz + qz;
                *internal_path += dist;
                pc->absorptions++;
                return 2;
            }
        }
        qx = tqx; qy = tqy; qz = tqz;
        *internal_path += chord;
        const float qn = sqrtf(qx * qx + qy * qy + qz * qz);
        if (!(qn > 0.0f) || !isfinite(qn)) { *pf = OP_MACRO_GEOMETRY; *pfs = OS_SPHERE_CHORD; return 0; }
        const float proj = rr / qn;
        qx *= proj; qy *= proj; qz *= proj;
        *x = cx + qx; *y = cy + qy; *z = cz + qz;
        float nox = qx / rr, noy = qy / rr, noz = qz / rr;
        o_normalize(&nox, &noy, &noz);
        const float bx = -nox, by = -noy, bz = -noz;
        top = 1; order = 0; mfc = OF_NONE;
        ms = o_micro_walk(s, rough_alpha, WD, bx, by, bz, n_particle, k_particle, n_medium, 0.0f, vx, vy, vz, &top,
                          &order, &mfc);
        *micro = order;
        if (ms != OM_ESCAPE) { *pf = (ms == OM_WATCHDOG) ? OP_MICRO_WATCHDOG : OP_MICRO_NUMERICAL; *pfs = mfc; return 0; }
        if (!top) {
            if (o_dot(*vx, *vy, *vz, nox, noy, noz) <= 0.0f) { *pf = OP_MACRO_GEOMETRY; *pfs = OS_SPHERE_EXIT_SIDE; return 0; }
            return 1;
        }
        if (o_dot(*vx, *vy, *vz, nox, noy, noz) >= 0.0f) { *pf = OP_MACRO_GEOMETRY; *pfs = OS_SPHERE_INTERNAL_SIDE; return 0; }
        pc->reflections++;
        pc->internal_reflections++;
        if (bounce == max_bounces) { *pf = OP_MACRO_BOUNCE_LIMIT; *pfs = OS_SPHERE_BOUNCE_LIMIT; return 0; }
    }
    *pf = OP_OTHER; *pfs = OS_NONE;
    return 0;
}
/* sphere interaction from a fresh placement at the origin (:2601-2612) */
template <class S>
__device__ int o_sphere_fresh(S* s, float n_medium, float n_particle, float k_particle, float wavelength,
                          float rough_alpha, float radius, int max_bounces, float* x, float* y, float* z, float* vx,
                          float* vy, float* vz, float* internal_path, o_pcount* pc, int* pf, int* pfs, int* macro,
                          int* micro, float* wmul = nullptr) {
    float rho, phi, gnx, gny, gnz;
    o_sphere_geometry(s, radius, *x, *y, *z, *vx, *vy, *vz, &rho, &phi, &gnx, &gny, &gnz);
    double cx = (double)(*x) - (double)radius * (double)gnx, cy = (double)(*y) - (double)radius * (double)gny,
           cz = (double)(*z) - (double)radius * (double)gnz;
    return o_sphere_sampled(s, n_medium, n_particle, k_particle, wavelength, rough_alpha, radius, max_bounces, gnx,
                            gny, gnz, cx, cy, cz, x, y, z, vx, vy, vz, internal_path, pc, pf, pfs, macro, micro, wmul);
}

/* Mie inverse-CDF angle (:2624-2652). The CDF comparisons are done after a float cast. */
template <class S>
__device__ __forceinline__ int o_sample_cdf(S* s, const float* cdf, int n) {
    if (n <= 1) return 0;
    float u = uniform(s);
    int lo = 0, hi = n - 1;
    while (lo < hi) { int mid = (lo + hi) >> 1; if (u <= cdf[mid]) hi = mid; else lo = mid + 1; }
    return lo;
}
template <class S>
__device__ __forceinline__ float o_mie_theta(S* s, const float* cdf, const float* theta, int nt, int pidx,
                                             const int* guide) {
    float u = uniform(s);
    int base = pidx * nt, lo = 0, hi = nt - 1;
    if (guide) {
        // u * kPhaseGuide is exact (a power of two): k/G <= u < (k+1)/G, so the first index with u <= cdf lies
        // between the first indices with cdf >= k/G and cdf >= (k+1)/G, and the search below finds it there
        const int k = min((int)(u * (float)kPhaseGuide), kPhaseGuide - 1);
        const int* g = guide + pidx * (kPhaseGuide + 1);
        lo = __ldg(g + k);
        hi = __ldg(g + k + 1);
    }
    while (lo < hi) { int mid = (lo + hi) >> 1; if (u <= __ldg(cdf + base + mid)) hi = mid; else lo = mid + 1; }
    int j = lo;
    if (j <= 0) return theta[0];
    float c0 = __ldg(cdf + base + j - 1), c1 = __ldg(cdf + base + j);
    float t0 = theta[j - 1], t1 = theta[j];
    float f = (c1 > c0) ? fminf(fmaxf((u - c0) / (c1 - c0), 0.0f), 1.0f) : 0.0f;
    return t0 + f * (t1 - t0);
}
template <class S>
__device__ __forceinline__ void o_mie_direction(S* s, const float* cdf, const float* theta, int nt, int pidx, float* vx,
                            float* vy, float* vz, const int* guide = nullptr) {
    float th = o_mie_theta(s, cdf, theta, nt, pidx, guide);
    float phi = 2.0f * CLR_PI_F * uniform(s);
    float e1x, e1y, e1z, e2x, e2y, e2z;
    o_perp_basis(*vx, *vy, *vz, &e1x, &e1y, &e1z, &e2x, &e2y, &e2z);
    float st = sinf(th), ct = cosf(th), cp = cosf(phi), sp = sinf(phi);
    float ox = ct * (*vx) + st * (cp * e1x + sp * e2x);
    float oy = ct * (*vy) + st * (cp * e1y + sp * e2y);
    float oz = ct * (*vz) + st * (cp * e1z + sp * e2z);
    *vx = ox; *vy = oy; *vz = oz;
    o_normalize(vx, vy, vz);
}

/* ---------------- spheroid morphology-wave event (:2660-2868) ---------------- */
template <class S>
__device__ void o_random_axis(S* s, float* ux, float* uy, float* uz) {
    float cz = 2.0f * uniform(s) - 1.0f;
    float az = 2.0f * CLR_PI_F * uniform(s);
    float sz = sqrtf(fmaxf(0.0f, 1.0f - cz * cz));
    *ux = sz * cosf(az); *uy = sz * sinf(az); *uz = cz;
}
template <class S>
__device__ void o_spheroid_axis(S* s, int model, float kappa, float fx, float fy, float fz, float* ux, float* uy,
                            float* uz) {
    if (model == 0 || !(kappa > 1e-7f) || !isfinite(kappa)) { o_random_axis(s, ux, uy, uz); return; }
    o_normalize(&fx, &fy, &fz);
    if (!(fx * fx + fy * fy + fz * fz > 0.5f)) { o_random_axis(s, ux, uy, uz); return; }
    float u = fminf(fmaxf(uniform(s), 1e-12f), 1.0f - 1e-7f);
    float em2 = expf(-2.0f * kappa);
    float c = 1.0f + logf(u + (1.0f - u) * em2) / kappa;
    c = fminf(fmaxf(c, -1.0f), 1.0f);
    float e1x, e1y, e1z, e2x, e2y, e2z;
    o_perp_basis(fx, fy, fz, &e1x, &e1y, &e1z, &e2x, &e2y, &e2z);
    float phi = 2.0f * CLR_PI_F * uniform(s);
    float st = sqrtf(fmaxf(0.0f, 1.0f - c * c));
    float cp = cosf(phi), sp = sinf(phi);
    *ux = c * fx + st * (cp * e1x + sp * e2x);
    *uy = c * fy + st * (cp * e1y + sp * e2y);
    *uz = c * fz + st * (cp * e1z + sp * e2z);
    if (uniform(s) < 0.5f) { *ux = -*ux; *uy = -*uy; *uz = -*uz; }
    o_normalize(ux, uy, uz);
}
__device__ __forceinline__ void o_spheroid_normal(float x, float y, float z, float ux, float uy, float uz, float invb2, float delta,
                                     float* nx, float* ny, float* nz) {
    float pu = x * ux + y * uy + z * uz;
    *nx = invb2 * x + delta * pu * ux;
    *ny = invb2 * y + delta * pu * uy;
    *nz = invb2 * z + delta * pu * uz;
    o_normalize(nx, ny, nz);
}
__device__ int o_spheroid_roots(float ox, float oy, float oz, float dx, float dy, float dz, float ux, float uy, float uz,
                            float invb2, float delta, float* t0, float* t1) {
    float du = dx * ux + dy * uy + dz * uz;
    float ou = ox * ux + oy * uy + oz * uz;
    float A = invb2 * (dx * dx + dy * dy + dz * dz) + delta * du * du;
    float B = 2.0f * (invb2 * (ox * dx + oy * dy + oz * dz) + delta * ou * du);
    float Cc = invb2 * (ox * ox + oy * oy + oz * oz) + delta * ou * ou - 1.0f;
    float disc = B * B - 4.0f * A * Cc;
    if (!(A > 0.0f) || disc < 0.0f) return 0;
    float sd = sqrtf(fmaxf(0.0f, disc));
    float r0 = (-B - sd) / (2.0f * A), r1 = (-B + sd) / (2.0f * A);
    if (r0 > r1) { float q = r0; r0 = r1; r1 = q; }
    *t0 = r0; *t1 = r1;
    return 1;
}
template <class S>
__device__ int o_spheroid_entry(S* s, float vx, float vy, float vz, float a, float b, float ux, float uy, float uz,
                            float* x, float* y, float* z, float* gnx, float* gny, float* gnz) {
    float invb2 = 1.0f / (b * b);
    float delta = 1.0f / (a * a) - invb2;
    float e1x, e1y, e1z, e2x, e2y, e2z;
    o_perp_basis(vx, vy, vz, &e1x, &e1y, &e1z, &e2x, &e2y, &e2z);
    float du = o_dot(ux, uy, uz, vx, vy, vz);
    float rproj2 = b * b + (a * a - b * b) * fmaxf(0.0f, 1.0f - du * du);
    float rbound = sqrtf(fmaxf(b * b, rproj2));
    float rmax = fmaxf(a, b);
    for (int attempt = 0; attempt < 64; ++attempt) {
        float rr = rbound * sqrtf(uniform(s));
        float ph = 2.0f * CLR_PI_F * uniform(s);
        float ox = rr * (cosf(ph) * e1x + sinf(ph) * e2x) - 2.5f * rmax * vx;
        float oy = rr * (cosf(ph) * e1y + sinf(ph) * e2y) - 2.5f * rmax * vy;
        float oz = rr * (cosf(ph) * e1z + sinf(ph) * e2z) - 2.5f * rmax * vz;
        float t0, t1;
        if (!o_spheroid_roots(ox, oy, oz, vx, vy, vz, ux, uy, uz, invb2, delta, &t0, &t1)) continue;
        float t = (t0 > 1e-9f * rmax) ? t0 : ((t1 > 1e-9f * rmax) ? t1 : -1.0f);
        if (t <= 0.0f) continue;
        *x = ox + t * vx; *y = oy + t * vy; *z = oz + t * vz;
        o_spheroid_normal(*x, *y, *z, ux, uy, uz, invb2, delta, gnx, gny, gnz);
        if (o_dot(vx, vy, vz, *gnx, *gny, *gnz) < -1e-6f) return 1;
    }
    return 0;
}
__device__ float o_spheroid_next(float x, float y, float z, float vx, float vy, float vz, float ux, float uy, float uz,
                             float invb2, float delta, float scale) {
    float t0, t1;
    if (!o_spheroid_roots(x, y, z, vx, vy, vz, ux, uy, uz, invb2, delta, &t0, &t1)) return -1.0f;
    float eps = fmaxf(1e-5f * scale, 1e-12f);
    float t = CLR_INF_F;
    if (t0 > eps) t = t0;
    if (t1 > eps && t1 < t) t = t1;
    return t < CLR_INF_F * 0.5f ? t : -1.0f;
}
/* direction-only spheroid (or sphere when q=1) event; 1 scattered, 2 absorbed, 0 failure (:2783-2849) */
template <class S>
__device__ __noinline__ int o_spheroid_event(S* s, float n_medium, float n_particle, float k_particle, float wavelength,
                            float rough_alpha, float r_equiv, float aspect, int orientation_model, float kappa,
                            float fx, float fy, float fz, int max_bounces, float* vx, float* vy, float* vz,
                            float* internal_path, o_pcount* pc, int* pf, int* pfs, int* macro, int* micro,
                            float* wmul = nullptr) {
    *pf = OP_OK; *pfs = OS_NONE; *macro = 0; *micro = 0;
    if (r_equiv <= 0.0f) return 1;
    if (!(aspect > 0.0f) || !isfinite(aspect)) { *pf = OP_SPHEROID_GEOMETRY; *pfs = OS_SPHEROID_ASPECT; return 0; }
    if (fabsf(aspect - 1.0f) < 1e-7f) {
        float lx = 0.0f, ly = 0.0f, lz = 0.0f, lvx = *vx, lvy = *vy, lvz = *vz, ip = 0.0f;
        int ps = o_sphere_fresh(s, n_medium, n_particle, k_particle, wavelength, rough_alpha, r_equiv, max_bounces, &lx,
                                &ly, &lz, &lvx, &lvy, &lvz, &ip, pc, pf, pfs, macro, micro, wmul);
        *internal_path += ip;
        if (ps == 1) { *vx = lvx; *vy = lvy; *vz = lvz; }
        return ps;
    }
    const int WD = 4096;
    float q13 = powf(aspect, 1.0f / 3.0f);
    float a = r_equiv * q13 * q13;
    float b = r_equiv / q13;
    if (!(a > 0.0f && b > 0.0f && isfinite(a) && isfinite(b))) { *pf = OP_SPHEROID_GEOMETRY; *pfs = OS_SPHEROID_AXES; return 0; }
    float ux, uy, uz;
    o_spheroid_axis(s, orientation_model, kappa, fx, fy, fz, &ux, &uy, &uz);
    float x, y, z, gnx, gny, gnz;
    if (!o_spheroid_entry(s, *vx, *vy, *vz, a, b, ux, uy, uz, &x, &y, &z, &gnx, &gny, &gnz)) {
        *pf = OP_SPHEROID_GEOMETRY; *pfs = OS_SPHEROID_ENTRY; return 0;
    }
    float invb2 = 1.0f / (b * b), delta = 1.0f / (a * a) - invb2, scale = fmaxf(a, b);
    int top = 1, order = 0, mfc = OF_NONE;
    int ms = o_micro_walk(s, rough_alpha, WD, gnx, gny, gnz, n_medium, 0.0f, n_particle, k_particle, vx, vy, vz, &top,
                          &order, &mfc);
    *micro = order;
    if (ms != OM_ESCAPE) { *pf = (ms == OM_WATCHDOG) ? OP_MICRO_WATCHDOG : OP_MICRO_NUMERICAL; *pfs = mfc; return 0; }
    if (top) { pc->reflections++; pc->entry_reflections++; return 1; }
    if (o_dot(*vx, *vy, *vz, gnx, gny, gnz) >= 0.0f) { *pf = OP_SPHEROID_GEOMETRY; *pfs = OS_SPHEROID_ENTRY; return 0; }
    float alpha_abs = (wavelength > 0.0f && k_particle > 0.0f) ? (4.0f * CLR_PI_F * k_particle / wavelength) : 0.0f;
    for (int bounce = 0; bounce <= max_bounces; ++bounce) {
        *macro = bounce;
        float chord = o_spheroid_next(x, y, z, *vx, *vy, *vz, ux, uy, uz, invb2, delta, scale);
        if (chord <= 0.0f) { *pf = OP_SPHEROID_GEOMETRY; *pfs = OS_SPHEROID_CHORD; return 0; }
        if (alpha_abs > 0.0f && wmul) {
            *wmul *= expf(-alpha_abs * chord);  // implicit capture: the chord's survival probability
        } else if (alpha_abs > 0.0f) {
            double dist = -log(open_uniform(s)) / (double)alpha_abs;
            if (dist < (double)chord) { *internal_path += (float)dist; pc->absorptions++; return 2; }
        }
        x += chord * (*vx); y += chord * (*vy); z += chord * (*vz);
        *internal_path += chord;
        float nox, noy, noz;
        o_spheroid_normal(x, y, z, ux, uy, uz, invb2, delta, &nox, &noy, &noz);
        float bx = -nox, by = -noy, bz = -noz;
        top = 1; order = 0; mfc = OF_NONE;
        ms = o_micro_walk(s, rough_alpha, WD, bx, by, bz, n_particle, k_particle, n_medium, 0.0f, vx, vy, vz, &top,
                          &order, &mfc);
        *micro = order;
        if (ms != OM_ESCAPE) { *pf = (ms == OM_WATCHDOG) ? OP_MICRO_WATCHDOG : OP_MICRO_NUMERICAL; *pfs = mfc; return 0; }
        if (!top) {
            if (o_dot(*vx, *vy, *vz, nox, noy, noz) <= 0.0f) { *pf = OP_SPHEROID_GEOMETRY; *pfs = OS_SPHEROID_EXIT_SIDE; return 0; }
            return 1;
        }
        if (o_dot(*vx, *vy, *vz, nox, noy, noz) >= 0.0f) { *pf = OP_SPHEROID_GEOMETRY; *pfs = OS_SPHEROID_INTERNAL_SIDE; return 0; }
        pc->reflections++;
        pc->internal_reflections++;
        if (bounce == max_bounces) { *pf = OP_MACRO_BOUNCE_LIMIT; *pfs = OS_SPHEROID_BOUNCE_LIMIT; return 0; }
    }
    *pf = OP_OTHER; *pfs = OS_NONE;
    return 0;
}

/* ---------------- acrylic solid, headspace, bottom disc (:2885-3293) ---------------- */
__device__ int o_cyl_roots(float x, float y, float vx, float vy, float R, double* t0, double* t1) {
    *t0 = 1.0e300; *t1 = 1.0e300;
    double X = (double)x, Y = (double)y, VX = (double)vx, VY = (double)vy, RR = (double)R;
    double a = VX * VX + VY * VY;
    if (!(a > 1e-30) || !isfinite(a)) return 0;
    double b = X * VX + Y * VY, c = X * X + Y * Y - RR * RR, d = b * b - a * c;
    double dscale = fabs(b * b) + fabs(a * c) + 1e-300;
    double dtol = 16.0 * CLR_DBL_EPS * dscale;
    if (d < 0.0) { if (d >= -dtol) d = 0.0; else return 0; }
    double sd = sqrt(fmax(d, 0.0)), q = -b - copysign(sd, b);
    double r0 = (fabs(q) > 1e-300) ? q / a : (-b - sd) / a;
    double r1 = (fabs(q) > 1e-300) ? c / q : (-b + sd) / a;
    double a0 = 1.0e300, a1 = 1.0e300;
    if (r0 > 0.0 && isfinite(r0)) a0 = r0;
    if (r1 > 0.0 && isfinite(r1)) { if (r1 < a0) { a1 = a0; a0 = r1; } else a1 = r1; }
    int n = 0;
    if (a0 < 1.0e299) n++;
    if (a1 < 1.0e299) n++;
    *t0 = a0; *t1 = a1;
    return n;
}
__device__ __forceinline__ double o_support_tol(float Rin, float Rout, float Zmin, float Zlow, float Ztop) {
    double scale = fmax(fmax(fabs((double)Rout), fabs((double)Zlow)), fabs((double)Ztop));
    scale = fmax(scale, fmax(fabs((double)Rin), fabs((double)Zmin)));
    return 8.0 * 1.1920928955078125e-7 * fmax(scale, 1.0e-3);
}
__device__ double o_cyl_hit_finite(float x, float y, float z, float vx, float vy, float vz, float R, float zlo, float zhi) {
    double r0, r1;
    o_cyl_roots(x, y, vx, vy, R, &r0, &r1);
    double tol = o_support_tol(R, R, zlo, zlo, zhi), best = 1.0e300;
    double roots[2] = {r0, r1};
    for (int k = 0; k < 2; ++k) {
        double t = roots[k];
        if (!(t > 0.0) || t >= 1.0e299) continue;
        double zh = (double)z + t * (double)vz;
        if (zh >= (double)zlo - tol && zh <= (double)zhi + tol && t < best) best = t;
    }
    return best;
}
__device__ double o_bore_wall_hit(float x, float y, float z, float vx, float vy, float vz, float R, float zlo, float zhi) {
    double X = x, Y = y, VX = vx, VY = vy, RR = (double)R * R;
    double rr2 = X * X + Y * Y, c = rr2 - RR, b = X * VX + Y * VY, a = VX * VX + VY * VY;
    double radial_tol = 8.0 * 1.1920928955078125e-7 * RR;
    double ztol = o_support_tol(R, R, zlo, zlo, zhi);
    if (c > radial_tol || !isfinite(c) || !isfinite(b) || !isfinite(a)) return -1.0;
    if (c >= 0.0) {
        if (b >= 0.0 && a > 0.0 && z >= zlo - ztol && z <= zhi + ztol) return 0.0;
        b *= sqrt(RR / rr2);
        c = 0.0;
    }
    if (!(a > 1e-30)) return 1.0e300;
    double d = b * b - a * c;
    if (d < 0.0) return 1.0e300;
    double sd = sqrt(d), q = -b - copysign(sd, b);
    double t = (b < 0.0) ? q / a : ((q != 0.0) ? c / q : 0.0);
    if (!(t >= 0.0) || !isfinite(t)) return 1.0e300;
    double zh = (double)z + t * (double)vz;
    return (zh >= zlo - ztol && zh <= zhi + ztol) ? t : 1.0e300;
}
/* FP32 distance to the tube wall from inside, for the counter-based stream: the same cases and
 * tolerances as o_bore_wall_hit (its tolerances are stated in FP32 epsilons already). */
__device__ __forceinline__ float f_bore_wall_hit(float x, float y, float z, float vx, float vy, float vz, float R,
                                                 float zlo, float zhi) {
    const float RR = R * R;
    const float rr2 = x * x + y * y;
    float c = rr2 - RR, b = x * vx + y * vy;
    const float a = vx * vx + vy * vy;
    const float radial_tol = 8.0f * 1.1920928955078125e-7f * RR;
    const float ztol = (float)o_support_tol(R, R, zlo, zlo, zhi);
    if (c > radial_tol || !isfinite(c) || !isfinite(b) || !isfinite(a)) return -1.0f;
    if (c >= 0.0f) {
        if (b >= 0.0f && a > 0.0f && z >= zlo - ztol && z <= zhi + ztol) return 0.0f;
        b *= sqrtf(RR / rr2);
        c = 0.0f;
    }
    if (!(a > 1e-30f)) return CLR_INF_F;
    const float d = b * b - a * c;
    if (d < 0.0f) return CLR_INF_F;
    const float sd = sqrtf(d), q = -b - copysignf(sd, b);
    const float t = (b < 0.0f) ? q / a : ((q != 0.0f) ? c / q : 0.0f);
    if (!(t >= 0.0f) || !isfinite(t)) return CLR_INF_F;
    const float zh = z + t * vz;
    return (zh >= zlo - ztol && zh <= zhi + ztol) ? t : CLR_INF_F;
}
/* water-side offset after a free-surface event (:2962-2977) */
__device__ int o_surface_offset(float* x, float* y, float* z, float nx, float ny, float nz, float R, float ZMIN,
                            float ZMEAN, int model, float dh, float core) {
    double rr2 = (double)(*x) * (double)(*x) + (double)(*y) * (double)(*y), RR = (double)R * R;
    double tol = 8.0 * 1.1920928955078125e-7 * RR;
    if (!isfinite(rr2) || rr2 > RR + tol) return 0;
    float xx = *x + CLR_EPS_F * nx, yy = *y + CLR_EPS_F * ny, zz = *z + CLR_EPS_F * nz;
    double rad = hypot((double)xx, (double)yy);
    if (rad > (double)R) {
        double target = (double)R * (1.0 - 2.0 * 1.1920928955078125e-7);
        xx = (float)((double)xx * target / rad);
        yy = (float)((double)yy * target / rad);
        float surf = o_surface_z(xx, yy, ZMEAN, R, model, dh, core);
        if (zz >= surf) zz = nextafterf(surf, -CLR_INF_F);
    }
    if (!isfinite(xx) || !isfinite(yy) || !isfinite(zz) || zz <= ZMIN || zz >= o_surface_z(xx, yy, ZMEAN, R, model, dh, core))
        return 0;
    *x = xx; *y = yy; *z = zz;
    return 1;
}
__device__ __forceinline__ void o_consider(double t, int surf, double* best, int* best_surf) {
    if (t > 0.0 && isfinite(t) && t < *best) { *best = t; *best_surf = surf; }
}
__device__ int o_acrylic_next(float x, float y, float z, float vx, float vy, float vz, float Rin, float Rout, float Zmin,
                          float Zlow, float Ztop, double* t_out) {
    double best = 1.0e300;
    int surf = 0;
    double tol = o_support_tol(Rin, Rout, Zmin, Zlow, Ztop);
    double r0, r1;
    o_cyl_roots(x, y, vx, vy, Rin, &r0, &r1);
    double ri[2] = {r0, r1};
    for (int k = 0; k < 2; ++k) {
        double t = ri[k];
        if (t >= 1.0e299) continue;
        double zh = (double)z + t * (double)vz;
        if (zh >= (double)Zmin - tol && zh <= (double)Ztop + tol) o_consider(t, 1, &best, &surf);
    }
    o_cyl_roots(x, y, vx, vy, Rout, &r0, &r1);
    double ro[2] = {r0, r1};
    for (int k = 0; k < 2; ++k) {
        double t = ro[k];
        if (t >= 1.0e299) continue;
        double zh = (double)z + t * (double)vz;
        if (zh >= (double)Zlow - tol && zh <= (double)Ztop + tol) o_consider(t, 2, &best, &surf);
    }
    if (vz < 0.0f) {
        double t = ((double)Zlow - (double)z) / (double)vz;
        if (t > 0.0 && isfinite(t)) {
            double X = (double)x + t * (double)vx, Y = (double)y + t * (double)vy, rr = hypot(X, Y);
            if (rr <= (double)Rout + tol) o_consider(t, 3, &best, &surf);
        }
    }
    if (vz > 0.0f) {
        double t = ((double)Ztop - (double)z) / (double)vz;
        if (t > 0.0 && isfinite(t)) {
            double X = (double)x + t * (double)vx, Y = (double)y + t * (double)vy, rr = hypot(X, Y);
            if (rr >= (double)Rin - tol && rr <= (double)Rout + tol) o_consider(t, 4, &best, &surf);
        }
        double ta = ((double)Zmin - (double)z) / (double)vz;
        if (ta > 0.0 && isfinite(ta)) {
            double X = (double)x + ta * (double)vx, Y = (double)y + ta * (double)vy, rr = hypot(X, Y);
            if (rr < (double)Rin - tol) o_consider(ta, 5, &best, &surf);
        }
    }
    *t_out = best;
    return surf;
}
__device__ __forceinline__ int o_tir_ci(double ci, double n1, double n2) {
    if (!(n1 > 0.0) || !(n2 > 0.0) || n1 <= n2) return 0;
    ci = fmin(fmax(ci, 0.0), 1.0);
    double st = (n1 / n2) * sqrt(fmax(0.0, 1.0 - ci * ci));
    return st >= 1.0;
}
/* ---- FP32 versions for the counter-based (production) stream ----
 * Same surfaces, same order of tests and the same support tolerance (already stated in FP32
 * epsilons); roots by the cancellation-free quadratic formula in FP32. Positions are FP32 in the
 * reference as well; the FP64 roots above are what the parity mode runs. */
__device__ __forceinline__ int f_cyl_roots(float x, float y, float vx, float vy, float R, float* t0, float* t1) {
    *t0 = CLR_INF_F; *t1 = CLR_INF_F;
    const float a = vx * vx + vy * vy;
    if (!(a > 1e-30f) || !isfinite(a)) return 0;
    const float b = x * vx + y * vy, c = (x * x + y * y) - R * R;
    float d = b * b - a * c;
    const float dtol = 16.0f * 1.1920928955078125e-7f * (fabsf(b * b) + fabsf(a * c) + 1e-30f);
    if (d < 0.0f) { if (d >= -dtol) d = 0.0f; else return 0; }
    const float sd = sqrtf(fmaxf(d, 0.0f)), q = -b - copysignf(sd, b);
    const float r0 = (fabsf(q) > 1e-30f) ? q / a : (-b - sd) / a;
    const float r1 = (fabsf(q) > 1e-30f) ? c / q : (-b + sd) / a;
    float a0 = CLR_INF_F, a1 = CLR_INF_F;
    if (r0 > 0.0f && isfinite(r0)) a0 = r0;
    if (r1 > 0.0f && isfinite(r1)) { if (r1 < a0) { a1 = a0; a0 = r1; } else a1 = r1; }
    *t0 = a0; *t1 = a1;
    return (a0 < CLR_INF_F) + (a1 < CLR_INF_F);
}
__device__ __forceinline__ void f_consider(float t, int surf, float* best, int* best_surf) {
    if (t > 0.0f && isfinite(t) && t < *best) { *best = t; *best_surf = surf; }
}
__device__ __forceinline__ int f_acrylic_next(float x, float y, float z, float vx, float vy, float vz, float Rin,
                                              float Rout, float Zmin, float Zlow, float Ztop, float* t_out) {
    float best = CLR_INF_F;
    int surf = 0;
    const float tol = (float)o_support_tol(Rin, Rout, Zmin, Zlow, Ztop);
    float r0, r1;
    f_cyl_roots(x, y, vx, vy, Rin, &r0, &r1);
    if (r0 < CLR_INF_F) { const float zh = z + r0 * vz; if (zh >= Zmin - tol && zh <= Ztop + tol) f_consider(r0, 1, &best, &surf); }
    if (r1 < CLR_INF_F) { const float zh = z + r1 * vz; if (zh >= Zmin - tol && zh <= Ztop + tol) f_consider(r1, 1, &best, &surf); }
    f_cyl_roots(x, y, vx, vy, Rout, &r0, &r1);
    if (r0 < CLR_INF_F) { const float zh = z + r0 * vz; if (zh >= Zlow - tol && zh <= Ztop + tol) f_consider(r0, 2, &best, &surf); }
    if (r1 < CLR_INF_F) { const float zh = z + r1 * vz; if (zh >= Zlow - tol && zh <= Ztop + tol) f_consider(r1, 2, &best, &surf); }
    if (vz < 0.0f) {
        const float t = (Zlow - z) / vz;
        if (t > 0.0f && isfinite(t)) {
            const float rr = hypotf(x + t * vx, y + t * vy);
            if (rr <= Rout + tol) f_consider(t, 3, &best, &surf);
        }
    }
    if (vz > 0.0f) {
        const float t = (Ztop - z) / vz;
        if (t > 0.0f && isfinite(t)) {
            const float rr = hypotf(x + t * vx, y + t * vy);
            if (rr >= Rin - tol && rr <= Rout + tol) f_consider(t, 4, &best, &surf);
        }
        const float ta = (Zmin - z) / vz;
        if (ta > 0.0f && isfinite(ta)) {
            const float rr = hypotf(x + ta * vx, y + ta * vy);
            if (rr < Rin - tol) f_consider(ta, 5, &best, &surf);
        }
    }
    *t_out = best;
    return surf;
}

/* conserved-orbit trapped-TIR classifier (:3089-3138) */
__device__ __noinline__ int o_trapped(float x, float y, float z, float vx, float vy, float vz, float n_water, float n_acrylic,
                     float n_air, float n_bottom_ext, float Rin, float Rout) {
    (void)z;
    double dx = (double)vx, dy = (double)vy, dz = (double)vz;
    double speed2 = dx * dx + dy * dy + dz * dz;
    if (!(speed2 > 0.0) || !isfinite(speed2)) return 0;
    double vxy2 = dx * dx + dy * dy;
    double L = (double)x * dy - (double)y * dx;
    double root_speed = sqrt(speed2);
    const double reach_tol = 4.0 * (double)CLR_EPS_F;
    if (vxy2 > 0.0) {
        double tang = L / (double)Rout;
        double rad2 = vxy2 - tang * tang;
        if (rad2 < 0.0 && rad2 > -1.0e-12 * speed2) rad2 = 0.0;
        if (rad2 < 0.0) return 0;
        double ci_outer = sqrt(rad2) / root_speed;
        if (!o_tir_ci(ci_outer, (double)n_acrylic, (double)n_air)) return 0;
        double impact = fabs(L) / sqrt(vxy2);
        if (impact <= (double)Rin + reach_tol) {
            double ti = L / (double)Rin;
            double ri2 = vxy2 - ti * ti;
            if (ri2 < 0.0 && ri2 > -1.0e-12 * speed2) ri2 = 0.0;
            if (ri2 >= 0.0) {
                double ci_inner = sqrt(ri2) / root_speed;
                if (!o_tir_ci(ci_inner, (double)n_acrylic, (double)n_water)) return 0;
            }
        }
        if (impact < (double)Rin - reach_tol && fabs(dz) > 0.0) {
            double ci_ax = fabs(dz) / root_speed;
            if (!o_tir_ci(ci_ax, (double)n_acrylic, (double)n_water)) return 0;
        }
    }
    if (fabs(dz) > 0.0) {
        double ci_ax = fabs(dz) / root_speed;
        if (vxy2 <= 1.0e-30 * speed2 && hypot((double)x, (double)y) < (double)Rin - reach_tol) {
            if (!o_tir_ci(ci_ax, (double)n_acrylic, (double)n_water)) return 0;
        }
        if (!o_tir_ci(ci_ax, (double)n_acrylic, (double)n_air)) return 0;
        if (!o_tir_ci(ci_ax, (double)n_acrylic, (double)n_bottom_ext)) return 0;
    }
    return 1;
}

typedef struct {
    int cir, cor, bir, bor, ctir, btir, tr, ttir;
} o_bcount;

typedef struct {
    float n_water, n_acrylic, n_air, n_bottom_ext;
    float Rin, Rout, Zmin, Zlow, Zmean, Ztop;
    int model; float dh, core;
} o_cell;

/* Bounces per window of the trapped-orbit test of long traversals (counter-based stream); the pieces a
 * traversal is cut into must start at multiples of 2 kTrapWindow. */
constexpr int kTrapWindow = 32;

/* Loop state of a traversal of the acrylic solid, so that a traversal can run in bounded pieces. */
typedef struct {
    int it, stuck, last_surf;
} o_acr_state;
__device__ __forceinline__ o_acr_state o_acr_start() {
    o_acr_state a = {0, 0, -1};
    return a;
}

/* inside the connected acrylic solid; 1 water, 2 external air, 3 bottom external, 4 headspace,
 * 5 trapped, 0 failure (:3143-3198). Runs bounces from as->it on; with budget > 0 at most `budget`
 * of them, returning -1 (and the loop state in *as) when the traversal has not ended by then. */
template <class S>
__device__ __noinline__ int o_acrylic_run(S* s, const o_cell* C, float n_side_air, float n_bottom_ext, float Zmin,
                                          float Zlow, float* x, float* y, float* z, float* vx, float* vy, float* vz,
                                          float* acrylic_path, o_bcount* bc, int* sub, int* out_bounces,
                                          o_acr_state* as, int budget) {
    const int cap = 16384;
    int stuck = as->stuck, last_surf = as->last_surf;
    const float n_water = C->n_water, n_acrylic = C->n_acrylic, n_air = n_side_air;
    const float Rin = C->Rin, Rout = C->Rout, Ztop = C->Ztop;
    const int it0 = as->it;
    const int end = (budget > 0 && cap - it0 > budget) ? it0 + budget : cap;
    int surf_next = 0;
    int it = it0;
    o_bcount snap = *bc;
    float snap_path = *acrylic_path;
    for (; it < end; ++it) {
        if constexpr (kCounterStream<S>) {
            // Counter-based stream only (no reference counterpart): a long traversal whose ray meets the
            // conserved-orbit trapped classifier (o_trapped: total internal reflection at every surface the
            // ray can reach, from invariants that reflection keeps) can never escape and ends trapped at the
            // bounce cap, as the classifier decides there. The remaining bounces are then accounted with the
            // reflection mix and path per bounce of the last kTrapWindow bounces, and the traversal goes
            // straight to the cap. The test runs at bounces it = (2k+1) kTrapWindow (it >= 512) only and its
            // window starts at a multiple of 2 kTrapWindow: pieces of a traversal start at multiples of that
            // too (budgets are multiples of it), so the window lies inside the running piece and the result
            // of a photon does not depend on how its traversal was cut into pieces.
            if ((it & (2 * kTrapWindow - 1)) == 0) {
                snap = *bc;
                snap_path = *acrylic_path;
            } else if (it >= 512 && (it & (2 * kTrapWindow - 1)) == kTrapWindow &&
                       o_trapped(*x, *y, *z, *vx, *vy, *vz, n_water, n_acrylic, n_air, n_bottom_ext, Rin, Rout)) {
                const long long left = cap - it;
                bc->cir += (int)((long long)(bc->cir - snap.cir) * left / kTrapWindow);
                bc->cor += (int)((long long)(bc->cor - snap.cor) * left / kTrapWindow);
                bc->bir += (int)((long long)(bc->bir - snap.bir) * left / kTrapWindow);
                bc->bor += (int)((long long)(bc->bor - snap.bor) * left / kTrapWindow);
                bc->ctir += (int)((long long)(bc->ctir - snap.ctir) * left / kTrapWindow);
                bc->btir += (int)((long long)(bc->btir - snap.btir) * left / kTrapWindow);
                *acrylic_path += (*acrylic_path - snap_path) * (float)((double)left / (double)kTrapWindow);
                it = cap;
                break;
            }
        }
        *out_bounces = it;
        float t;
        if constexpr (kCounterStream<S>) {
            int surf_f = f_acrylic_next(*x, *y, *z, *vx, *vy, *vz, Rin, Rout, Zmin, Zlow, Ztop, &t);
            if (!surf_f || !(t > 0.0f) || !isfinite(t) || t >= CLR_INF_F) { *sub = OS_ACRYLIC_NO_INTERSECTION; return 0; }
            surf_next = surf_f;
        } else {
            double td = 1.0e300;
            int surf_d = o_acrylic_next(*x, *y, *z, *vx, *vy, *vz, Rin, Rout, Zmin, Zlow, Ztop, &td);
            if (!surf_d || !(td > 0.0) || !isfinite(td) || td >= 1.0e299) { *sub = OS_ACRYLIC_NO_INTERSECTION; return 0; }
            t = (float)td;
            surf_next = surf_d;
        }
        const int surf = surf_next;
        float px = *x, py = *y, pz = *z, pvx = *vx, pvy = *vy, pvz = *vz;
        *x += t * (*vx); *y += t * (*vy); *z += t * (*vz);
        *acrylic_path += t;
        float a, b, c;
        int tir = 0;
        float ci = 0.0f, R = 1.0f;
        if (surf == 1) {
            float nx, ny;
            o_radial_normal(*x, *y, &nx, &ny);
            float zs = o_surface_z(*x, *y, C->Zmean, Rin, C->model, C->dh, C->core);
            float n_in = ((*z <= zs + CLR_EPS_F) ? n_water : n_air);
            ci = fminf(fmaxf(-o_dot(*vx, *vy, *vz, nx, ny, 0.0f), 0.0f), 1.0f);
            R = o_fresnel(ci, n_acrylic, n_in, &tir);
            if (!tir && uniform(s) >= R && o_refract(*vx, *vy, *vz, nx, ny, 0.0f, n_acrylic, n_in, &a, &b, &c)) {
                *vx = a; *vy = b; *vz = c; *x -= CLR_EPS_F * nx; *y -= CLR_EPS_F * ny;
                return (n_in == n_water) ? 1 : 4;
            }
            o_reflect(*vx, *vy, *vz, nx, ny, 0.0f, &a, &b, &c);
            *vx = a; *vy = b; *vz = c; bc->cir++; if (tir) bc->ctir++;
            *x += CLR_EPS_F * nx; *y += CLR_EPS_F * ny;
        } else if (surf == 2) {
            float nx, ny;
            o_radial_normal(*x, *y, &nx, &ny);
            ci = fminf(fmaxf(o_dot(*vx, *vy, *vz, nx, ny, 0.0f), 0.0f), 1.0f);
            R = o_fresnel(ci, n_acrylic, n_air, &tir);
            if (!tir && uniform(s) >= R && o_refract(*vx, *vy, *vz, -nx, -ny, 0.0f, n_acrylic, n_air, &a, &b, &c)) {
                *vx = a; *vy = b; *vz = c; *x += CLR_EPS_F * nx; *y += CLR_EPS_F * ny;
                return 2;
            }
            o_reflect(*vx, *vy, *vz, nx, ny, 0.0f, &a, &b, &c);
            *vx = a; *vy = b; *vz = c; bc->cor++; if (tir) bc->ctir++;
            *x -= CLR_EPS_F * nx; *y -= CLR_EPS_F * ny;
        } else if (surf == 3) {
            *z = Zlow;
            ci = fminf(fmaxf(-(*vz), 0.0f), 1.0f);
            R = o_fresnel(ci, n_acrylic, n_bottom_ext, &tir);
            if (!tir && uniform(s) >= R && o_refract(*vx, *vy, *vz, 0.0f, 0.0f, 1.0f, n_acrylic, n_bottom_ext, &a, &b, &c)) {
                *vx = a; *vy = b; *vz = c; *z = Zlow - CLR_EPS_F;
                return 3;
            }
            o_reflect(*vx, *vy, *vz, 0.0f, 0.0f, 1.0f, &a, &b, &c);
            *vx = a; *vy = b; *vz = c; bc->bor++; if (tir) bc->btir++;
            *z = Zlow + CLR_EPS_F;
        } else if (surf == 4) {
            *z = Ztop;
            ci = fminf(fmaxf(*vz, 0.0f), 1.0f);
            R = o_fresnel(ci, n_acrylic, n_air, &tir);
            if (!tir && uniform(s) >= R && o_refract(*vx, *vy, *vz, 0.0f, 0.0f, -1.0f, n_acrylic, n_air, &a, &b, &c)) {
                *vx = a; *vy = b; *vz = c; *z = Ztop + CLR_EPS_F;
                return 2;
            }
            o_reflect(*vx, *vy, *vz, 0.0f, 0.0f, 1.0f, &a, &b, &c);
            *vx = a; *vy = b; *vz = c; bc->cor++; if (tir) bc->ctir++;
            *z = Ztop - CLR_EPS_F;
        } else if (surf == 5) {
            *z = Zmin;
            ci = fminf(fmaxf(*vz, 0.0f), 1.0f);
            R = o_fresnel(ci, n_acrylic, n_water, &tir);
            if (!tir && uniform(s) >= R && o_refract(*vx, *vy, *vz, 0.0f, 0.0f, -1.0f, n_acrylic, n_water, &a, &b, &c)) {
                *vx = a; *vy = b; *vz = c; *z = Zmin + CLR_EPS_F;
                return 1;
            }
            o_reflect(*vx, *vy, *vz, 0.0f, 0.0f, 1.0f, &a, &b, &c);
            *vx = a; *vy = b; *vz = c; bc->bir++; if (tir) bc->btir++;
            *z = Zmin - CLR_EPS_F;
        } else {
            *sub = OS_ACRYLIC_NO_INTERSECTION;
            return 0;
        }
        float pd = fabsf(*x - px) + fabsf(*y - py) + fabsf(*z - pz);
        float vd = fabsf(*vx - pvx) + fabsf(*vy - pvy) + fabsf(*vz - pvz);
        stuck = (surf == last_surf && pd <= 1.0e-12f && vd <= 1.0e-7f) ? (stuck + 1) : 0;
        if (stuck >= 8) { *sub = OS_ACRYLIC_BOUNCE_LIMIT; return 0; }
        last_surf = surf;
    }
    if (it < cap) {  // the budget ran out first (it == end)
        as->it = it; as->stuck = stuck; as->last_surf = last_surf;
        return -1;
    }
    if (o_trapped(*x, *y, *z, *vx, *vy, *vz, n_water, n_acrylic, n_air, n_bottom_ext, Rin, Rout)) {
        *sub = OS_NONE; *out_bounces = 16384;
        return 5;
    }
    *sub = OS_ACRYLIC_BOUNCE_LIMIT;
    *out_bounces = 16384;
    return 0;
}
template <class S>
__device__ __forceinline__ int o_acrylic_solid(S* s, const o_cell* C, float n_side_air, float n_bottom_ext, float Zmin,
                                               float Zlow, float* x, float* y, float* z, float* vx, float* vy,
                                               float* vz, float* acrylic_path, o_bcount* bc, int* sub,
                                               int* out_bounces) {
    *sub = OS_NONE;
    *out_bounces = 0;
    o_acr_state as = o_acr_start();
    return o_acrylic_run(s, C, n_side_air, n_bottom_ext, Zmin, Zlow, x, y, z, vx, vy, vz, acrylic_path, bc, sub,
                         out_bounces, &as, 0);
}
/* water -> bottom disc (:3211-3224), first part: 1 reflected back into the water, 0 failure,
 * 6 transmitted into the disc (the traversal of the acrylic solid follows) */
template <class S>
__device__ __forceinline__ int o_bottom_entry(S* s, const o_cell* C, float* x, float* y, float* z, float* vx,
                                              float* vy, float* vz, o_bcount* bc, int* sub, int* out_bounces) {
    *sub = OS_NONE;
    *out_bounces = 0;
    {
        double r2 = (double)(*x) * (double)(*x) + (double)(*y) * (double)(*y);
        double ri2 = (double)C->Rin * (double)C->Rin;
        if (!(r2 < ri2)) { *sub = OS_BOTTOM_TOPOLOGY; return 0; }
    }
    float a, b, c;
    int tir = 0;
    float ci = fminf(fmaxf(-o_dot(*vx, *vy, *vz, 0.0f, 0.0f, 1.0f), 0.0f), 1.0f);
    float R = o_fresnel(ci, C->n_water, C->n_acrylic, &tir);
    if (tir || uniform(s) < R || !o_refract(*vx, *vy, *vz, 0.0f, 0.0f, 1.0f, C->n_water, C->n_acrylic, &a, &b, &c)) {
        o_reflect(*vx, *vy, *vz, 0.0f, 0.0f, 1.0f, &a, &b, &c);
        *vx = a; *vy = b; *vz = c; bc->bir++; if (tir) bc->btir++;
        *z = C->Zmin + CLR_EPS_F;
        return 1;
    }
    *vx = a; *vy = b; *vz = c;
    *z = C->Zmin - CLR_EPS_F;
    return 6;
}
template <class S>
__device__ __noinline__ int o_bottom_disc(S* s, const o_cell* C, float* x, float* y, float* z, float* vx, float* vy, float* vz,
                         float* acrylic_path, o_bcount* bc, int* sub, int* out_bounces) {
    const int e = o_bottom_entry(s, C, x, y, z, vx, vy, vz, bc, sub, out_bounces);
    if (e != 6) return e;
    return o_acrylic_solid(s, C, C->n_air, C->n_bottom_ext, C->Zmin, C->Zlow, x, y, z, vx, vy, vz, acrylic_path, bc,
                           sub, out_bounces);
}
/* headspace above the free surface; 1 water, 2 external, 3 bottom external, 4 open top,
 * 5 trapped, 0 failure (:3235-3293) */
template <class S>
__device__ __noinline__ int o_headspace(S* s, const o_cell* C, float* x, float* y, float* z, float* vx, float* vy, float* vz,
                       float* acrylic_path, o_bcount* bc, int* sub, int* out_bounces) {
    *sub = OS_NONE;
    *out_bounces = 0;
    const int cap = 16384;
    const float Rin = C->Rin, Zmin = C->Zmin, Ztop = C->Ztop;
    double tol = o_support_tol(Rin, C->Rout, Zmin, C->Zlow, Ztop);
    for (int step = 0; step < cap; ++step) {
        *out_bounces = step;
        if (!isfinite(*x) || !isfinite(*y) || !isfinite(*z) || !isfinite(*vx) || !isfinite(*vy) || !isfinite(*vz)) {
            *sub = OS_HEADSPACE_NO_BOUNDARY; return 0;
        }
        float zs = o_surface_z(*x, *y, C->Zmean, Rin, C->model, C->dh, C->core);
        double rr = hypot((double)*x, (double)*y);
        if ((double)*z <= (double)zs - tol && rr < (double)Rin - tol) return 1;
        if ((double)*z > (double)Ztop + tol) return 4;
        double tside = o_bore_wall_hit(*x, *y, *z, *vx, *vy, *vz, Rin, Zmin, Ztop);
        if (tside < 0.0) { *sub = OS_WATER_OUTSIDE; return 0; }
        double tsurf = (double)o_surface_hit(*x, *y, *z, *vx, *vy, *vz, C->Zmean, Rin, C->model, C->dh, C->core);
        double ttop = 1.0e300;
        if (*vz > 1.0e-14f) {
            double t = ((double)Ztop - (double)*z) / (double)*vz;
            if (t > 0.0) {
                double X = (double)*x + t * (double)*vx, Y = (double)*y + t * (double)*vy;
                if (hypot(X, Y) < (double)Rin + tol) ttop = t;
            }
        }
        int which = 0;
        double best = 1.0e300;
        if (tsurf > 0.0 && tsurf < best) { best = tsurf; which = 1; }
        if (tside >= 0.0 && tside < best) { best = tside; which = 2; }
        if (ttop > 0.0 && ttop < best) { best = ttop; which = 3; }
        if (!which || !isfinite(best) || best >= 1.0e299) { *sub = OS_HEADSPACE_NO_BOUNDARY; return 0; }
        float t = (float)best;
        *x += t * (*vx); *y += t * (*vy); *z += t * (*vz);
        if (which == 3) { *z = Ztop + CLR_EPS_F; return 4; }
        float a, b, c;
        int tir = 0;
        if (which == 1) {
            float snx, sny, snz;
            o_surface_normal(*x, *y, Rin, C->model, C->dh, C->core, &snx, &sny, &snz);
            float anx = -snx, any = -sny, anz = -snz;
            float ci = fminf(fmaxf(-o_dot(*vx, *vy, *vz, anx, any, anz), 0.0f), 1.0f);
            float R = o_fresnel(ci, C->n_air, C->n_water, &tir);
            if (tir || uniform(s) < R || !o_refract(*vx, *vy, *vz, anx, any, anz, C->n_air, C->n_water, &a, &b, &c)) {
                o_reflect(*vx, *vy, *vz, anx, any, anz, &a, &b, &c);
                *vx = a; *vy = b; *vz = c; bc->tr++; if (tir) bc->ttir++;
                *x += CLR_EPS_F * anx; *y += CLR_EPS_F * any; *z += CLR_EPS_F * anz;
                continue;
            }
            *vx = a; *vy = b; *vz = c;
            if (!o_surface_offset(x, y, z, snx, sny, snz, Rin, Zmin, C->Zmean, C->model, C->dh, C->core)) {
                *sub = OS_WATER_OUTSIDE; return 0;
            }
            return 1;
        }
        float nx, ny;
        o_radial_normal(*x, *y, &nx, &ny);
        float inx = -nx, iny = -ny;
        float ci = fminf(fmaxf(-o_dot(*vx, *vy, *vz, inx, iny, 0.0f), 0.0f), 1.0f);
        float R = o_fresnel(ci, C->n_air, C->n_acrylic, &tir);
        if (tir || uniform(s) < R || !o_refract(*vx, *vy, *vz, inx, iny, 0.0f, C->n_air, C->n_acrylic, &a, &b, &c)) {
            o_reflect(*vx, *vy, *vz, inx, iny, 0.0f, &a, &b, &c);
            *vx = a; *vy = b; *vz = c; bc->cir++; if (tir) bc->ctir++;
            *x -= CLR_EPS_F * nx; *y -= CLR_EPS_F * ny;
            continue;
        }
        *vx = a; *vy = b; *vz = c;
        *x += CLR_EPS_F * nx; *y += CLR_EPS_F * ny;
        int asub = OS_NONE, ab = 0;
        int where = o_acrylic_solid(s, C, C->n_air, C->n_bottom_ext, C->Zmin, C->Zlow, x, y, z, vx, vy, vz,
                                    acrylic_path, bc, &asub, &ab);
        if (where == 4) continue;
        *sub = asub;
        *out_bounces = ab;
        return where;
    }
    *sub = OS_HEADSPACE_NO_BOUNDARY;
    *out_bounces = cap;
    return 0;
}

}  // namespace
}  // namespace clr
