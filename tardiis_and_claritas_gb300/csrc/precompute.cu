// Particle-physics precompute on the device (FP64).
//
// Replaces the precompute launched by ClaritasForwardModel._prepare_gpu_particle_physics
// (CLARITAS/CLARITAS.py:6036-6965). The per-bin and per-angle arithmetic is the
// reference's (kernels :3488-3592, :3845-3921, :3925-4038), so the tables the
// photon kernel reads are identical to the reference's on the same GPU; only
// the parallel decomposition changes:
//  * Mie coefficients: one warp per size bin, the downward log-derivative
//    recurrence kept in shared memory instead of a global scratch array;
//  * phase pdf: one thread per (angle, group of 4 bins) sharing the angular
//    pi_n/tau_n recurrence across the group (the recurrence depends only on the
//    angle), instead of one thread per (bin, angle) recomputing it;
//  * Schiller-Naumann radial slip: one thread per (bin, radius) instead of one
//    thread for everything; the serial prefix sums and quadrature stay serial
//    per bin so their rounding is unchanged.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include "kernels.h"

namespace clr {

#define PD_PI 3.141592653589793238462643383279502884

struct cdx { double re, im; };
__device__ __forceinline__ cdx CD(double re, double im) { cdx z; z.re = re; z.im = im; return z; }
__device__ __forceinline__ cdx cd_add(cdx a, cdx b) { return CD(a.re + b.re, a.im + b.im); }
__device__ __forceinline__ cdx cd_sub(cdx a, cdx b) { return CD(a.re - b.re, a.im - b.im); }
__device__ __forceinline__ cdx cd_mul(cdx a, cdx b) { return CD(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
__device__ __forceinline__ cdx cd_scale(cdx a, double s) { return CD(a.re * s, a.im * s); }
__device__ __forceinline__ cdx cd_div(cdx a, cdx b) {
    double d = b.re * b.re + b.im * b.im;
    if (d < 1e-300) d = 1e-300;
    return CD((a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d);
}
__device__ __forceinline__ double cd_abs2(cdx a) { return a.re * a.re + a.im * a.im; }
__device__ __forceinline__ double cd_rmc(cdx a, cdx b) { return a.re * b.re + a.im * b.im; }

// One warp per bin (:3495-3559). The recurrences are serial and stay on lane 0: the downward
// log-derivative recurrence D_{n-1} = n/z - 1/(D_n + n/z) and the upward Riccati-Bessel psi/chi
// recurrences. Everything independent across orders is spread over the 32 lanes: the n/z quotients
// before the downward recurrence, and the a_n, b_n quotients after it. The efficiency sums stay
// serial on lane 0. Every value has the one-thread expression, and every sum its order.
// Shared memory: D[0..nmx], n/z[0..nmx] (complex) and psi[0..nstop+1], chi[0..nstop+1] (real), laid out
// for `order_cap` orders (at most CLR_MIE_MAX_ORDER; a launch over small particles asks for less, so more
// blocks share an SM). The a_n, b_n rows of `ab` are `order_cap` orders apart.
__host__ __device__ constexpr size_t mie_smem_bytes(int order_cap) {
    return (size_t)2 * (order_cap + 1) * sizeof(cdx) + (size_t)2 * (order_cap + 2) * sizeof(double);
}
constexpr size_t kMieSmem = mie_smem_bytes(CLR_MIE_MAX_ORDER);

__global__ void __launch_bounds__(32) mie_coefficients_kernel(const double* __restrict__ diameter,
                                                              const double* __restrict__ n_real,
                                                              const double* __restrict__ k_imag, double n_medium,
                                                              double wavelength, int n_particles, int order_cap,
                                                              double* __restrict__ ab, int* __restrict__ nstop_out,
                                                              double* size_parameter, double* qext, double* qsca,
                                                              double* qabs, double* qback, double* asym_g,
                                                              double* albedo, int* error_flag) {
    extern __shared__ cdx Dsh[];
    cdx* NZ = Dsh + (order_cap + 1);
    double* PSI = reinterpret_cast<double*>(NZ + (order_cap + 1));
    double* CHI = PSI + (order_cap + 2);
    const int p = blockIdx.x;
    const int lane = threadIdx.x;
    if (p >= n_particles) return;
    double x = PD_PI * n_medium * diameter[p] / wavelength;
    if (!(x > 0.0) || !(n_real[p] > 0.0) || !(n_medium > 0.0) || !(wavelength > 0.0)) {
        if (lane == 0) {
            size_parameter[p] = x;
            nstop_out[p] = 0; qext[p] = qsca[p] = qabs[p] = qback[p] = asym_g[p] = 0.0; albedo[p] = 1.0;
            atomicCAS(error_flag, 0, 2);
        }
        return;
    }
    double mr = n_real[p] / n_medium, mi = k_imag[p] / n_medium;
    int nstop = (int)(x + 4.0 * cbrt(x) + 2.0);
    if (nstop < 1) nstop = 1;
    double mz = hypot(mr * x, mi * x);
    int nmx = (int)fmax((double)nstop, mz) + 128;
    if (nmx < nstop + 1) nmx = nstop + 1;
    if (nmx >= CLR_MIE_MAX_ORDER || nstop >= CLR_MIE_MAX_ORDER) {
        if (lane == 0) { size_parameter[p] = x; nstop_out[p] = 0; atomicCAS(error_flag, 0, 1); }
        return;
    }
    if (nmx > order_cap) {  // the host's bound on the orders of this launch was too small (never expected)
        if (lane == 0) { size_parameter[p] = x; nstop_out[p] = 0; atomicCAS(error_flag, 0, CLR_ERR_CODE_ORDER_CAP); }
        return;
    }
    const cdx z = CD(mr * x, mi * x);
    for (int n = 1 + lane; n <= nmx; n += 32) NZ[n] = cd_div(CD((double)n, 0.0), z);
    __syncwarp();
    if (lane == 0) {
        size_parameter[p] = x;
        nstop_out[p] = nstop;
        Dsh[nmx] = CD(0.0, 0.0);
        for (int n = nmx; n >= 1; --n) {
            cdx nz = NZ[n];
            cdx dn = Dsh[n];
            Dsh[n - 1] = cd_sub(nz, cd_div(CD(1.0, 0.0), cd_add(dn, nz)));
        }
    }
    __syncwarp();
    // (2n+1)/x of every order, in the n/z space (no longer needed), for the upward recurrences
    double* Q2X = reinterpret_cast<double*>(NZ);
    for (int n = 1 + lane; n <= nstop; n += 32) Q2X[n] = (2.0 * n + 1.0) / x;
    __syncwarp();
    if (lane == 0) {
        double psi_nm1 = sin(x), psi_n = sin(x) / x - cos(x);
        double chi_nm1 = cos(x), chi_n = cos(x) / x + sin(x);
        PSI[0] = psi_nm1; PSI[1] = psi_n; CHI[0] = chi_nm1; CHI[1] = chi_n;
        for (int n = 1; n <= nstop; ++n) {
            double psi_np1 = Q2X[n] * psi_n - psi_nm1;
            double chi_np1 = Q2X[n] * chi_n - chi_nm1;
            psi_nm1 = psi_n; psi_n = psi_np1; chi_nm1 = chi_n; chi_n = chi_np1;
            PSI[n + 1] = psi_n; CHI[n + 1] = chi_n;
        }
    }
    __syncwarp();
    const cdx m = CD(mr, mi);
    double4* abp = reinterpret_cast<double4*>(ab) + (size_t)p * order_cap;
    for (int j = lane; j < nstop; j += 32) {
        int n = j + 1;
        const double psi_nm1 = PSI[n - 1], psi_n = PSI[n], chi_nm1 = CHI[n - 1], chi_n = CHI[n];
        cdx xi_nm1 = CD(psi_nm1, -chi_nm1), xi_n = CD(psi_n, -chi_n);
        cdx dn = Dsh[n];
        cdx ca = cd_add(cd_div(dn, m), CD((double)n / x, 0.0));
        cdx cb = cd_add(cd_mul(m, dn), CD((double)n / x, 0.0));
        cdx aa = cd_div(cd_sub(cd_scale(ca, psi_n), CD(psi_nm1, 0.0)), cd_sub(cd_mul(ca, xi_n), xi_nm1));
        cdx bb = cd_div(cd_sub(cd_scale(cb, psi_n), CD(psi_nm1, 0.0)), cd_sub(cd_mul(cb, xi_n), xi_nm1));
        abp[j] = make_double4(aa.re, aa.im, bb.re, bb.im);
    }
    // quotients of the efficiency sums, in the same space (Q2X is no longer needed):
    // C1[n] = (2n+1)/(n(n+1)), C2[n] = n(n+2)/(n+1)
    double* C1 = Q2X;
    double* C2 = Q2X + (order_cap + 1);
    for (int n = 1 + lane; n <= nstop; n += 32) {
        const double cn = 2.0 * n + 1.0;
        C1[n] = cn / ((double)n * (n + 1.0));
        C2[n] = (double)n * (n + 2.0) / (n + 1.0);
    }
    __syncwarp();
    if (lane != 0) return;
    double se = 0.0, ss = 0.0, sbr = 0.0, sbi = 0.0, t1 = 0.0, t2 = 0.0;
    for (int j = 0; j < nstop; ++j) {
        int n = j + 1;
        double cn = 2.0 * n + 1.0;
        double4 q = abp[j];
        cdx aa = CD(q.x, q.y), bb = CD(q.z, q.w);
        se += cn * (aa.re + bb.re);
        ss += cn * (cd_abs2(aa) + cd_abs2(bb));
        double sign = (n & 1) ? -1.0 : 1.0;
        sbr += cn * sign * (aa.re - bb.re);
        sbi += cn * sign * (aa.im - bb.im);
        t2 += C1[n] * cd_rmc(aa, bb);
        if (j + 1 < nstop) {
            double4 q2 = abp[j + 1];
            cdx an = CD(q2.x, q2.y), bn = CD(q2.z, q2.w);
            t1 += C2[n] * (cd_rmc(aa, an) + cd_rmc(bb, bn));
        }
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
    qext[p] = qe; qsca[p] = qs; qabs[p] = qa; qback[p] = qb; asym_g[p] = gg; albedo[p] = qe > 0.0 ? qs / qe : 1.0;
}

// theta_j = pi/2 (1 - cos(pi j/(nt-1))) (:3488-3493), plus the float copy the sampler reads
__global__ void theta_grid_kernel(double* theta, float* theta_f, int nt) {
    int j = blockDim.x * blockIdx.x + threadIdx.x;
    if (j >= nt) return;
    double v;
    if (j == 0) v = 0.0;
    else if (j == nt - 1) v = PD_PI;
    else { double u = (double)j / (double)(nt - 1); v = 0.5 * PD_PI * (1.0 - cos(PD_PI * u)); }
    theta[j] = v;
    theta_f[j] = (float)v;
}

#define PDF_GROUP 4
__host__ __device__ constexpr size_t pdf_smem_bytes(int order_cap) { return (size_t)order_cap * sizeof(double3); }
constexpr size_t kPdfSmem = pdf_smem_bytes(CLR_MIE_MAX_ORDER);
// S1/S2 -> 0.5(|S1|^2+|S2|^2) sin(theta) for PDF_GROUP bins at one angle (:3561-3581)
__global__ void __launch_bounds__(128) phase_pdf_kernel(const double* __restrict__ theta, int nt, int n_particles,
                                                        int order_cap, const int* __restrict__ nstop,
                                                        const double* __restrict__ ab, double* __restrict__ pdf) {
    // quotients of each order n = k + 1 (identical to evaluating them inline):
    // (2n+1)/(n(n+1)), (2n+1)/n, (n+1)/n
    extern __shared__ double3 QN[];  // [order_cap], dynamic (pdf_smem_bytes(order_cap))
    const int j = blockDim.x * blockIdx.x + threadIdx.x;
    const int g0 = blockIdx.y * PDF_GROUP;
    int kmax_blk = 0;
    for (int g = 0; g < PDF_GROUP; ++g)
        if (g0 + g < n_particles && nstop[g0 + g] > kmax_blk) kmax_blk = nstop[g0 + g];
    for (int k = threadIdx.x; k < kmax_blk; k += blockDim.x) {
        const double nf = (double)(k + 1);
        QN[k] = make_double3((2.0 * nf + 1.0) / (nf * (nf + 1.0)), (2.0 * nf + 1.0) / nf, (nf + 1.0) / nf);
    }
    __syncthreads();
    if (j >= nt) return;
    double th = theta[j], mu = cos(th);
    double s1r[PDF_GROUP], s1i[PDF_GROUP], s2r[PDF_GROUP], s2i[PDF_GROUP];
    int ns[PDF_GROUP];
    int kmax = 0;
#pragma unroll
    for (int g = 0; g < PDF_GROUP; ++g) {
        s1r[g] = s1i[g] = s2r[g] = s2i[g] = 0.0;
        ns[g] = (g0 + g < n_particles) ? nstop[g0 + g] : 0;
        kmax = ns[g] > kmax ? ns[g] : kmax;
    }
    const double4* abp = reinterpret_cast<const double4*>(ab);
    double pi_nm1 = 0.0, pi_n = 1.0;
    for (int k = 0; k < kmax; ++k) {
        int n = k + 1;
        double nf = (double)n;
        double tau = nf * mu * pi_n - (nf + 1.0) * pi_nm1;
        const double3 qn = QN[k];  // the three quotients of order n, computed once per block above
        double c = qn.x;
#pragma unroll
        for (int g = 0; g < PDF_GROUP; ++g) {
            if (k < ns[g]) {
                double4 q = abp[(size_t)(g0 + g) * order_cap + k];
                double ar = q.x, ai = q.y, br = q.z, bi = q.w;
                s1r[g] += c * (ar * pi_n + br * tau);
                s1i[g] += c * (ai * pi_n + bi * tau);
                s2r[g] += c * (ar * tau + br * pi_n);
                s2i[g] += c * (ai * tau + bi * pi_n);
            }
        }
        double pi_np1 = qn.y * mu * pi_n - qn.z * pi_nm1;
        pi_nm1 = pi_n; pi_n = pi_np1;
    }
#pragma unroll
    for (int g = 0; g < PDF_GROUP; ++g) {
        if (g0 + g < n_particles) {
            double intensity = 0.5 * (s1r[g] * s1r[g] + s1i[g] * s1i[g] + s2r[g] * s2r[g] + s2i[g] * s2i[g]);
            pdf[(size_t)(g0 + g) * nt + j] = intensity * sin(th);
        }
    }
}

// Production variant of the phase pdf (CLR_TABLES_FAST; no reference counterpart). The same S1/S2 sums,
// evaluated with fused multiply-adds on coefficients premultiplied by (2n+1)/(n(n+1)) (staged per block in
// shared memory), and for two angles at once: theta_j and theta_{nt-1-j}, which is pi - theta_j on the
// reference's grid to rounding. With pi_n(-mu) = (-1)^(n-1) pi_n(mu) and tau_n(-mu) = (-1)^n tau_n(mu), the
// sums over odd and over even orders of a pi_n, b tau_n, a tau_n and b pi_n give S1 and S2 at mu and at
// -mu: 8 FMAs per (bin, order) for both angles, against about 44 FP64 operations of the reference's order
// of operations for the two. Tables differ from the reference-order ones by rounding only (tested).
constexpr int kPdfFastGroup = 4;    // bins per block (one Legendre recurrence per angle serves them all)
constexpr int kPdfFastChunk = 128;  // orders staged per block
__global__ void __launch_bounds__(128) phase_pdf_fast_kernel(const double* __restrict__ theta, int nt,
                                                             int n_particles, int order_cap,
                                                             const int* __restrict__ nstop,
                                                             const double* __restrict__ ab, double* __restrict__ pdf) {
    __shared__ double4 AB[kPdfFastGroup][kPdfFastChunk];
    __shared__ double2 RC[kPdfFastChunk];  // (2n+1)/n, (n+1)/n of the staged orders
    const int g0 = blockIdx.y * kPdfFastGroup;
    const int npair = (nt + 1) / 2;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = j < npair;
    int ns[kPdfFastGroup];
    int kmax = 0;
#pragma unroll
    for (int g = 0; g < kPdfFastGroup; ++g) {
        ns[g] = (g0 + g < n_particles) ? nstop[g0 + g] : 0;
        kmax = ns[g] > kmax ? ns[g] : kmax;
    }
    const double mu = active ? cos(theta[j]) : 0.0;
    // per bin: odd-order sums P = a pi, Q = b tau, R = a tau, T = b pi (re, im), then the even-order ones
    double acc[kPdfFastGroup][16];
#pragma unroll
    for (int g = 0; g < kPdfFastGroup; ++g)
#pragma unroll
        for (int i = 0; i < 16; ++i) acc[g][i] = 0.0;
    const double4* ab4 = reinterpret_cast<const double4*>(ab);
    double pi_nm1 = 0.0, pi_n = 1.0;
    for (int k0 = 0; k0 < kmax; k0 += kPdfFastChunk) {
        __syncthreads();
        for (int idx = threadIdx.x; idx < kPdfFastGroup * kPdfFastChunk; idx += blockDim.x) {
            const int g = idx / kPdfFastChunk, kk = idx % kPdfFastChunk, k = k0 + kk;
            double4 v = make_double4(0.0, 0.0, 0.0, 0.0);
            if (k < ns[g]) {
                const double4 q = ab4[(size_t)(g0 + g) * order_cap + k];
                const double nf = (double)(k + 1);
                const double c = (2.0 * nf + 1.0) / (nf * (nf + 1.0));
                v = make_double4(c * q.x, c * q.y, c * q.z, c * q.w);
            }
            AB[g][kk] = v;
        }
        for (int kk = threadIdx.x; kk < kPdfFastChunk; kk += blockDim.x) {
            const double nf = (double)(k0 + kk + 1);
            RC[kk] = make_double2((2.0 * nf + 1.0) / nf, (nf + 1.0) / nf);
        }
        __syncthreads();
        const int kend = min(kPdfFastChunk, kmax - k0);
        // k0 is even, so order n = k0 + kk + 1 is odd for even kk: odd-order sums go to acc[g][0..7], even-order
        // ones to acc[g][8..15]; the pair loop keeps every index a compile-time constant (registers, no stack).
        // Orders past kend carry zero coefficients, so the pair's second half may run past it.
        for (int kk = 0; kk < kend; kk += 2) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const double nf = (double)(k0 + kk + h + 1);
                const double tau = fma(nf * mu, pi_n, -(nf + 1.0) * pi_nm1);
#pragma unroll
                for (int g = 0; g < kPdfFastGroup; ++g) {
                    const double4 q = AB[g][kk + h];
                    double* A = acc[g] + 8 * h;
                    A[0] = fma(q.x, pi_n, A[0]); A[1] = fma(q.y, pi_n, A[1]);  // P
                    A[2] = fma(q.z, tau, A[2]);  A[3] = fma(q.w, tau, A[3]);   // Q
                    A[4] = fma(q.x, tau, A[4]);  A[5] = fma(q.y, tau, A[5]);   // R
                    A[6] = fma(q.z, pi_n, A[6]); A[7] = fma(q.w, pi_n, A[7]);  // T
                }
                const double2 rc = RC[kk + h];
                const double pi_np1 = fma(rc.x * mu, pi_n, -rc.y * pi_nm1);
                pi_nm1 = pi_n; pi_n = pi_np1;
            }
        }
    }
    if (!active) return;
    const int jm = nt - 1 - j;
    const double sj = sin(theta[j]), sm = sin(theta[jm]);
#pragma unroll
    for (int g = 0; g < kPdfFastGroup; ++g) {
        if (g0 + g >= n_particles) continue;
        const double* o = acc[g];
        const double* e = acc[g] + 8;
        // S1(mu) = Po+Qo+Pe+Qe, S1(-mu) = Po-Qo-Pe+Qe, S2(mu) = Ro+To+Re+Te, S2(-mu) = -Ro+To+Re-Te
        const double s1r = o[0] + o[2] + e[0] + e[2], s1i = o[1] + o[3] + e[1] + e[3];
        const double s2r = o[4] + o[6] + e[4] + e[6], s2i = o[5] + o[7] + e[5] + e[7];
        pdf[(size_t)(g0 + g) * nt + j] = 0.5 * (s1r * s1r + s1i * s1i + s2r * s2r + s2i * s2i) * sj;
        if (jm != j) {
            const double m1r = o[0] - o[2] - e[0] + e[2], m1i = o[1] - o[3] - e[1] + e[3];
            const double m2r = -o[4] + o[6] + e[4] - e[6], m2i = -o[5] + o[7] + e[5] - e[7];
            pdf[(size_t)(g0 + g) * nt + jm] = 0.5 * (m1r * m1r + m1i * m1i + m2r * m2r + m2i * m2i) * sm;
        }
    }
}

// Trapezoid CDF per bin, normalised and forced monotone (:3583-3592); also the float copy. One warp per
// bin: the trapezoid areas and the normalised values are independent per angle and spread over the
// lanes; the prefix sum and the monotone clamp stay serial on lane 0, so every value is the serial one.
__global__ void __launch_bounds__(32) phase_cdf_kernel(const double* __restrict__ theta, const double* __restrict__ pdf,
                                                       int nt, int n_particles, double* __restrict__ cdf,
                                                       float* __restrict__ cdf_f, int* error_flag) {
    const int p = blockIdx.x;
    const int lane = threadIdx.x;
    if (p >= n_particles) return;
    const long long base = (long long)p * nt;
    for (int j = 1 + lane; j < nt; j += 32) {
        double area = 0.5 * (pdf[base + j] + pdf[base + j - 1]) * (theta[j] - theta[j - 1]);
        if (area < 0.0 && area > -1e-18) area = 0.0;
        cdf[base + j] = area;
    }
    __syncwarp();
    double s = 0.0;
    if (lane == 0) {
        cdf[base] = 0.0;
        for (int j = 1; j < nt; ++j) {
            s += cdf[base + j];
            cdf[base + j] = s;
        }
    }
    s = __shfl_sync(0xffffffffu, s, 0);
    __syncwarp();
    if (!(s > 0.0) || !isfinite(s)) {
        if (lane == 0) atomicCAS(error_flag, 0, 3);
        for (int j = lane; j < nt; j += 32) { cdf[base + j] = (double)j / (double)(nt - 1); cdf_f[base + j] = (float)cdf[base + j]; }
        return;
    }
    for (int j = lane; j < nt; j += 32) cdf[base + j] = cdf[base + j] / s;
    __syncwarp();
    if (lane == 0) {
        double prev = 0.0;
        for (int j = 0; j < nt; ++j) {
            double v = cdf[base + j];
            if (v < prev) v = prev;
            if (v > 1.0) v = 1.0;
            cdf[base + j] = v;
            prev = v;
        }
        cdf[base + nt - 1] = 1.0;
    }
    __syncwarp();
    for (int j = lane; j < nt; j += 32) cdf_f[base + j] = (float)cdf[base + j];
}

// guide[p][k] = the first index j of bin p with cdf_f[j] >= k / kPhaseGuide (nt - 1 when none), found by the
// photon kernels' own search, so that a search restricted to [guide[k], guide[k+1]] returns its index
__global__ void phase_guide_kernel(const float* __restrict__ cdf_f, int nt, int n_particles, int* __restrict__ guide) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n_particles * (kPhaseGuide + 1)) return;
    const int p = (int)(t / (kPhaseGuide + 1)), k = (int)(t % (kPhaseGuide + 1));
    const float u = (float)k / (float)kPhaseGuide;
    const float* c = cdf_f + (size_t)p * nt;
    int lo = 0, hi = nt - 1;
    while (lo < hi) { const int mid = (lo + hi) >> 1; if (u <= c[mid]) hi = mid; else lo = mid + 1; }
    guide[t] = lo;
}

__global__ void dummy_phase_kernel(double* theta, float* theta_f, double* cdf, float* cdf_f, int n_particles) {
    int p = blockDim.x * blockIdx.x + threadIdx.x;
    if (p == 0) { theta[0] = 0.0; theta[1] = PD_PI; theta_f[0] = 0.0f; theta_f[1] = (float)PD_PI; }
    if (p < n_particles) { cdf[2 * p] = 0.0; cdf[2 * p + 1] = 1.0; cdf_f[2 * p] = 0.0f; cdf_f[2 * p + 1] = 1.0f; }
}

// PSD normalisation (:3615-3635), rates and channel CDFs (:3845-3921), channel rate arrays
// (:6362-6375) and the float copies the photon kernel reads. n <= 64: one thread.
__device__ __noinline__ void transport_body(int n, const double* __restrict__ d, const double* __restrict__ w_in,
                                            const double* __restrict__ qext, const double* __restrict__ qsca,
                                            const double* __restrict__ k_imag, const double* __restrict__ n_real,
                                            double concentration, double density, int weight_mode, int em,
                                            double wave_scale, double n_medium, double wavelength, double wave_rms,
                                            double* w, double* radius, double* nden, double* mug, double* mus,
                                            double* mue, double* muw, double* muev, double* gcdf, double* wcdf,
                                            double* pcdf, double* muscal, double* trace_geom, double* trace_wave,
                                            float* gcdf_f, float* wcdf_f, float* pn_f, float* pk_f, float* prad_f,
                                            int* error_flag) {
    if (n < 1 || n > CLR_MAX_BINS) { atomicCAS(error_flag, 0, 20); return; }
    if (!(density > 0.0) || concentration < 0.0) { atomicCAS(error_flag, 0, 21); return; }
    double sw0 = 0.0;
    for (int i = 0; i < n; ++i) sw0 += w_in[i];
    if (!(sw0 > 0.0)) { atomicCAS(error_flag, 0, 22); return; }
    for (int i = 0; i < n; ++i) w[i] = w_in[i] / sw0;
    double sw = 0.0;
    for (int i = 0; i < n; ++i) sw += w[i];
    if (!(sw > 0.0)) { atomicCAS(error_flag, 0, 4); return; }
    double pmass[CLR_MAX_BINS], srcw[CLR_MAX_BINS];
    double avg_mass = 0.0;
    for (int i = 0; i < n; ++i) {
        double r = 0.5 * d[i];
        radius[i] = r;
        srcw[i] = w[i] / sw;
        double m = density * (4.0 / 3.0) * PD_PI * r * r * r;
        pmass[i] = m;
        avg_mass += srcw[i] * m;
    }
    for (int i = 0; i < n; ++i) {
        double nd = 0.0;
        if (weight_mode == 0) nd = concentration * srcw[i] / pmass[i];
        else nd = (avg_mass > 0.0 ? concentration / avg_mass : 0.0) * srcw[i];
        nden[i] = nd;
        double sg = PD_PI * radius[i] * radius[i], sa = fmax(qsca[i], 0.0) * sg, se = fmax(qext[i], 0.0) * sg;
        double tol = 1e-10 * fmax(1.0, fmax(fabs(qext[i]), fabs(qsca[i])));
        const double ki = k_imag[i];
        if (!isfinite(ki) || ki < 0.0 || !isfinite(qext[i]) || !isfinite(qsca[i]) || qext[i] < -tol || qsca[i] < -tol ||
            qsca[i] > qext[i] + tol || (ki == 0.0 && fabs(qext[i] - qsca[i]) > tol)) {
            atomicCAS(error_flag, 0, 5);
            return;
        }
        double swv = 0.0;
        if (em == 3) swv = wave_scale * fmax(qsca[i] - 1.0, 0.0) * sg;
        else if (em == 4 || em == 5) {
            double rate = (ki > 0.0) ? se : sa;
            swv = (ki > 0.0) ? ((sa > 0.0) ? rate * fmax(sa - sg, 0.0) / sa : 0.0) : fmax(sa - sg, 0.0);
        }
        mug[i] = nd * sg; mus[i] = nd * sa; mue[i] = nd * se; muw[i] = nd * swv;
    }
    double mg = 0.0, ms = 0.0, me = 0.0, mw = 0.0;
    for (int i = 0; i < n; ++i) { mg += mug[i]; ms += mus[i]; me += mue[i]; mw += muw[i]; }
    double mt = 0.0;
    for (int i = 0; i < n; ++i) {
        double mb;
        if (em == 0) mb = mug[i];
        else if (em == 1) mb = mus[i];
        else if (em == 2) mb = mue[i];
        else if (em == 3) mb = mug[i] + muw[i];
        else mb = (k_imag[i] > 0.0) ? mue[i] : mus[i];
        muev[i] = mb;
        mt += mb;
    }
    const bool hyb = (em == 3) || (em == 4) || (em == 5);
    double mtrace_geom = ((em == 4) || (em == 5)) ? fmax(mt - mw, 0.0) : ((em == 3) ? mg : mt);
    double mtrace_wave = hyb ? mw : 0.0;
    double cg = 0.0, cw = 0.0, ct = 0.0;
    for (int i = 0; i < n; ++i) {
        double mgi = ((em == 4) || (em == 5)) ? fmax(muev[i] - muw[i], 0.0) : mug[i];
        double pg = hyb ? (mtrace_geom > 0.0 ? mgi / mtrace_geom : 0.0) : (mt > 0.0 ? muev[i] / mt : 0.0);
        double pw = (hyb && mtrace_wave > 0.0 ? muw[i] / mtrace_wave : 0.0), pt = (mt > 0.0 ? muev[i] / mt : 0.0);
        cg += pg; cw += pw; ct += pt;
        gcdf[i] = cg; wcdf[i] = cw; pcdf[i] = ct;
    }
    if (cg > 0.0) gcdf[n - 1] = 1.0;
    if (cw > 0.0) wcdf[n - 1] = 1.0;
    if (ct > 0.0) pcdf[n - 1] = 1.0;
    muscal[0] = mtrace_geom; muscal[1] = mtrace_wave; muscal[2] = mg; muscal[3] = ms;
    muscal[4] = me; muscal[5] = mtrace_wave; muscal[6] = mt;
    double cwave = 1.0;
    if (hyb && wave_rms > 0.0 && wavelength > 0.0 && n_medium > 0.0) {
        double a = 4.0 * PD_PI * n_medium * wave_rms / wavelength;
        cwave = exp(-a * a);
        if (cwave < 0.0) cwave = 0.0;
        if (cwave > 1.0) cwave = 1.0;
    }
    muscal[7] = cwave;
    for (int i = 0; i < n; ++i) {
        if (em == 3) { trace_geom[i] = mug[i]; trace_wave[i] = muw[i]; }
        else if (em == 4 || em == 5) { trace_geom[i] = fmax(muev[i] - muw[i], 0.0); trace_wave[i] = muw[i]; }
        else { trace_geom[i] = muev[i]; trace_wave[i] = 0.0; }
        gcdf_f[i] = (float)gcdf[i];
        wcdf_f[i] = (float)wcdf[i];
        pn_f[i] = (float)n_real[i];
        pk_f[i] = (float)k_imag[i];
        prad_f[i] = (float)radius[i];
    }
}

// The rates of one scenario (a single thread) and of many scenarios in one launch (a thread per
// scenario): both run transport_body, so every value is the same.
struct TransportJob {
    int n, weight_mode, em;
    const double *d, *w_in, *qext, *qsca, *k_imag, *n_real;
    double concentration, density, wave_scale, n_medium, wavelength, wave_rms;
    double *w, *radius, *nden, *mug, *mus, *mue, *muw, *muev, *gcdf, *wcdf, *pcdf, *muscal, *trace_geom, *trace_wave;
    float *gcdf_f, *wcdf_f, *pn_f, *pk_f, *prad_f;
    int* error_flag;
};
__device__ __forceinline__ void transport_job(const TransportJob& j) {
    transport_body(j.n, j.d, j.w_in, j.qext, j.qsca, j.k_imag, j.n_real, j.concentration, j.density, j.weight_mode,
                   j.em, j.wave_scale, j.n_medium, j.wavelength, j.wave_rms, j.w, j.radius, j.nden, j.mug, j.mus,
                   j.mue, j.muw, j.muev, j.gcdf, j.wcdf, j.pcdf, j.muscal, j.trace_geom, j.trace_wave, j.gcdf_f,
                   j.wcdf_f, j.pn_f, j.pk_f, j.prad_f, j.error_flag);
}
__global__ void transport_kernel(TransportJob j) {
    if (blockIdx.x || threadIdx.x) return;
    transport_job(j);
}
__global__ void transport_batch_kernel(const TransportJob* __restrict__ jobs, int count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) transport_job(jobs[i]);
}

// Schiller-Naumann terminal velocity by damped Newton (:3925-3937)
__device__ double sn_velocity(double v0, double d, double rho_w, double mu, double* out_Re, double* out_drag) {
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

struct SedArgs {
    int n, TM, FSM, NQ, NRAD;
    double rho_p, rho_w, mu, grav, Dt, R, ZMIN, ZMEAN, DH, CORE;
};

__device__ __forceinline__ void sed_geometry(const SedArgs& a, double* R2, double* a2, double* Hinf, double* hbar,
                                             double* omega2, double* fR) {
    *R2 = a.R * a.R; *a2 = a.CORE * a.CORE; *Hinf = 0.0; *hbar = 0.0; *omega2 = 0.0;
    if (a.DH > 0.0 && a.FSM == 1) { *Hinf = a.DH; *hbar = 0.5 * a.DH; *omega2 = 2.0 * a.grav * a.DH / *R2; }
    else if (a.DH > 0.0 && a.FSM == 2) {
        *Hinf = a.DH * (*a2 + *R2) / *R2;
        *hbar = *Hinf * (1.0 - (*a2 / *R2) * log1p(*R2 / *a2));
        *omega2 = 2.0 * a.grav * *Hinf / *a2;
    }
    *fR = (a.FSM == 2) ? *R2 / (*a2 + *R2) : *R2;
}

// Per-bin radial slip table: one thread per (bin, radius) for the finite-Re models (:3975-3986).
__global__ void sediment_slip_kernel(SedArgs a, const double* __restrict__ diameter, double* __restrict__ wr_out) {
    const int i = blockIdx.y;
    const int j = blockDim.x * blockIdx.x + threadIdx.x;
    if (i >= a.n || j >= a.NRAD || a.TM == 0 || a.TM == 1) return;
    double R2, a2, Hinf, hbar, omega2, fR;
    sed_geometry(a, &R2, &a2, &Hinf, &hbar, &omega2, &fR);
    double d = diameter[i];
    double tau = a.rho_p * d * d / (18.0 * a.mu);
    double drad = a.R / (double)(a.NRAD - 1);
    double r = (double)j * drad, acc = 0.0;
    if (r > 0.0) acc = (a.FSM == 1) ? omega2 * r : ((a.FSM == 2) ? omega2 * r / pow(1.0 + r * r / a2, 2.0) : 0.0);
    double w0 = tau * acc, re = 0.0, drag = 1.0;
    wr_out[(size_t)i * a.NRAD + j] = sn_velocity(w0, d, a.rho_w, a.mu, &re, &drag);
}

// Per-bin coefficients, radial potential and normalisation (:3958-4035); one warp per bin. Lane 0 runs
// the serial parts (slip velocity, prefix sums of the radial potential, the quadrature sum); the
// quadrature terms, each an independent exp/expm1 evaluation, are computed by all lanes into `terms`
// first, so every value and the order of every sum are those of the one-thread version.
__global__ void __launch_bounds__(32) sediment_bin_kernel(SedArgs a, const double* __restrict__ diameter,
                                                          const double* __restrict__ wr, double* sedA, double* sedB,
                                                          double* sed_norm, double* sed_max, double* radial_log,
                                                          double* __restrict__ terms, double* ws_out,
                                                          int* error_flag) {
    const int i = blockIdx.x;
    const int lane = threadIdx.x;
    if (i >= a.n) return;
    if (a.TM == 0) {
        if (lane == 0) { sedA[i] = 0.0; sedB[i] = 0.0; sed_norm[i] = 1.0; sed_max[i] = 1.0; ws_out[i] = 0.0; }
        return;
    }
    double R2, a2, Hinf, hbar, omega2, fR;
    sed_geometry(a, &R2, &a2, &Hinf, &hbar, &omega2, &fR);
    const double R = a.R, ZMIN = a.ZMIN, ZMEAN = a.ZMEAN, DH = a.DH;
    const int NRAD = a.NRAD, NQ = a.NQ, FSM = a.FSM, TM = a.TM;
    double Hmean = ZMEAN - ZMIN, dr = R / (double)NQ, drad = R / (double)(NRAD - 1);
    double d = diameter[i];
    double tau = a.rho_p * d * d / (18.0 * a.mu);
    double ws0 = (a.rho_p - a.rho_w) * a.grav * d * d / (18.0 * a.mu);
    double sre = 0.0, sdrag = 1.0;
    double ws = (TM == 2 || TM == 3) ? sn_velocity(ws0, d, a.rho_w, a.mu, &sre, &sdrag) : ws0;
    double Bc = ws / a.Dt;
    double* RL = radial_log + (size_t)i * NRAD;
    const double Ac = tau * omega2 * ((FSM == 2) ? a2 : 1.0) / (2.0 * a.Dt);
    if (lane == 0) {
        sedB[i] = Bc;
        ws_out[i] = ws;
        if (TM == 1) {
            sedA[i] = Ac;
            for (int j = 0; j < NRAD; ++j) {
                double r = (double)j * drad, rr2 = r * r, f = (FSM == 2) ? rr2 / (a2 + rr2) : rr2;
                RL[j] = Ac * (f - fR);
            }
        } else {
            const double* W = wr + (size_t)i * NRAD;
            double total = 0.0, prev = 0.0;
            for (int j = 0; j < NRAD; ++j) {
                double w = W[j];
                if (j > 0) total += 0.5 * (prev + w) * drad;
                prev = w;
            }
            double cum = 0.0;
            prev = 0.0;
            for (int j = 0; j < NRAD; ++j) {
                double w = W[j];
                if (j > 0) cum += 0.5 * (prev + w) * drad;
                prev = w;
                double psi = (cum - total) / a.Dt;
                if (psi > 0.0) psi = 0.0;
                RL[j] = psi;
            }
            RL[NRAD - 1] = 0.0;
            sedA[i] = (fR > 0.0) ? -RL[0] / fR : 0.0;
        }
    }
    __syncwarp();
    const double A_i = (TM == 1) ? Ac : ((fR > 0.0) ? -RL[0] / fR : 0.0);
    double* T = terms + (size_t)i * NQ;
    for (int j = lane; j < NQ; j += 32) {
        double r = ((double)j + 0.5) * dr, rr2 = r * r;
        double zsurf = ZMEAN;
        if (FSM == 1 && DH > 0.0) zsurf = ZMEAN + DH * (rr2 / R2 - 0.5);
        else if (FSM == 2 && DH > 0.0) zsurf = ZMEAN - hbar + Hinf * rr2 / (a2 + rr2);
        double Hh = fmax(zsurf - ZMIN, 0.0);
        double rl;
        if (TM == 1) {
            double f = (FSM == 2) ? rr2 / (a2 + rr2) : rr2;
            rl = A_i * (f - fR);
        } else {
            double u = r / R * (double)(NRAD - 1);
            int k = (int)floor(u);
            if (k < 0) k = 0;
            if (k > NRAD - 2) k = NRAD - 2;
            double t = u - (double)k;
            rl = (1.0 - t) * RL[k] + t * RL[k + 1];
            if (rl > 0.0) rl = 0.0;
        }
        double radial = exp(rl);
        double iz = (fabs(Bc) < 1e-14) ? radial * Hh : radial * (-expm1(-Bc * Hh)) / Bc;
        T[j] = r * iz;
    }
    __syncwarp();
    if (lane != 0) return;
    double integ = 0.0;
    for (int j = 0; j < NQ; ++j) integ += T[j];
    double norm = (2.0 / (R2 * Hmean)) * integ * dr;
    if (!(norm > 0.0) || !isfinite(norm)) { atomicCAS(error_flag, 0, 34); return; }
    sed_norm[i] = norm;
    sed_max[i] = 1.0 / norm;
}

// Per-bin maximum of the (r, z) grid (the max of non-negative terms starting at 0, as the reference's
// serial scan, so the order of the reduction does not change the value). One block per bin.
__global__ void sediment_grid_max_kernel(const double* __restrict__ grid, long long plane, double* grid_max) {
    const int p = blockIdx.x;
    double mx = 0.0;
    for (long long c = threadIdx.x; c < plane; c += blockDim.x) {
        const double q = grid[p * plane + c];
        if (q > mx) mx = q;
    }
    __shared__ double red[256];
    red[threadIdx.x] = mx;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h && red[threadIdx.x + h] > red[threadIdx.x]) red[threadIdx.x] = red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) grid_max[p] = red[0];
}

__device__ __noinline__ void majorant_body(const SedArgs& a, const double* trace_geom, const double* trace_wave,
                                           double* sed_A, double* sed_norm, double* sed_max, const double* grid_max,
                                           double* major, int* error_flag) {
    const int n = a.n;
    double mg = 0.0, mw = 0.0;
    if (a.TM == 0) {
        for (int i = 0; i < n; ++i) { mg += trace_geom[i]; mw += trace_wave[i]; }
        major[0] = mg; major[1] = mw; major[2] = mg + mw; major[3] = 0.0;
        return;
    }
    double maxAeq = 0.0;
    for (int i = 0; i < n; ++i) {
        if (sed_A[i] > maxAeq) maxAeq = sed_A[i];
        mg += trace_geom[i] * sed_max[i];
        mw += trace_wave[i] * sed_max[i];
    }
    major[0] = mg; major[1] = mw; major[2] = mg + mw; major[3] = maxAeq;
    if (!(major[2] >= 0.0) || !isfinite(major[2])) atomicCAS(error_flag, 0, 35);
    if (a.TM == 3 && grid_max) {
        for (int p = 0; p < n; ++p) {
            double mx = grid_max[p];
            if (!(mx > 0.0)) mx = 1.0;
            sed_norm[p] = 1.0;
            sed_max[p] = mx;
        }
        mg = 0.0; mw = 0.0;
        for (int i = 0; i < n; ++i) { mg += trace_geom[i] * sed_max[i]; mw += trace_wave[i] * sed_max[i]; }
        major[0] = mg; major[1] = mw; major[2] = mg + mw;
    }
}

struct MajorantJob {
    SedArgs a;
    const double *trace_geom, *trace_wave, *grid_max;
    double *sed_A, *sed_norm, *sed_max, *major;
    int* error_flag;
};
__global__ void sediment_majorant_kernel(MajorantJob j) {
    if (blockIdx.x || threadIdx.x) return;
    majorant_body(j.a, j.trace_geom, j.trace_wave, j.sed_A, j.sed_norm, j.sed_max, j.grid_max, j.major, j.error_flag);
}
__global__ void sediment_majorant_batch_kernel(const MajorantJob* __restrict__ jobs, int count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) {
        const MajorantJob& j = jobs[i];
        majorant_body(j.a, j.trace_geom, j.trace_wave, j.sed_A, j.sed_norm, j.sed_max, j.grid_max, j.major,
                      j.error_flag);
    }
}

// Node tables of the (r, z) field for the counter-based stream: for channel ch (0 geometric, 1 wave) and
// node c, G = sum_i mu_ch[i] grid[i][c] (FP64, bin order) and a Walker/Vose alias table over the bins with
// probabilities mu_ch[i] grid[i][c] / G. One thread per (channel, node); reads of grid[i][c] coalesce over c.
// The host enables these tables only for grids with no negative value, where the reference's clamp of the
// interpolated value at zero never acts, so the interpolated sum equals the interpolation of the sums.
__global__ void sediment_node_kernel(const double* __restrict__ grid, const double* __restrict__ trace_geom,
                                     const double* __restrict__ trace_wave, int n, int plane, float2* node_mu,
                                     int2* node_alias, unsigned int* node_major_bits) {
    const int t = blockDim.x * blockIdx.x + threadIdx.x;
    if (t >= 2 * plane) return;
    const int ch = t / plane, c = t - ch * plane;
    const double* mu = ch ? trace_wave : trace_geom;
    double p[CLR_MAX_BINS];
    double G = 0.0;
    for (int i = 0; i < n; ++i) {
        p[i] = mu[i] * grid[(size_t)i * plane + c];
        G += p[i];
    }
    float* dst = reinterpret_cast<float*>(&node_mu[c]) + ch;
    *dst = (float)G;
    int2* A = node_alias + ((size_t)ch * plane + c) * n;
    if (!(G > 0.0)) {
        for (int i = 0; i < n; ++i) A[i] = make_int2(__float_as_int(1.0f), i);
    } else {
        unsigned char small[CLR_MAX_BINS], large[CLR_MAX_BINS];
        int ns = 0, nl = 0;
        for (int i = 0; i < n; ++i) {
            p[i] = p[i] * (double)n / G;
            if (p[i] < 1.0) small[ns++] = (unsigned char)i; else large[nl++] = (unsigned char)i;
        }
        while (ns > 0 && nl > 0) {
            const int sm = small[--ns], lg = large[--nl];
            A[sm] = make_int2(__float_as_int((float)p[sm]), lg);
            p[lg] = (p[lg] + p[sm]) - 1.0;
            if (p[lg] < 1.0) small[ns++] = (unsigned char)lg; else large[nl++] = (unsigned char)lg;
        }
        while (nl > 0) { const int i = large[--nl]; A[i] = make_int2(__float_as_int(1.0f), i); }
        while (ns > 0) { const int i = small[--ns]; A[i] = make_int2(__float_as_int(1.0f), i); }
    }
    if (ch == 0) {
        // majorant of the summed field: max over nodes of G_geom + G_wave (non-negative, so the
        // float bit patterns order like the values)
        double Gw = 0.0;
        for (int i = 0; i < n; ++i) Gw += trace_wave[i] * grid[(size_t)i * plane + c];
        const float tot = (float)(G + Gw) * (1.0f + 4.0f * 1.1920928955078125e-7f);
        atomicMax(node_major_bits, __float_as_uint(tot));
    }
}

// ---------------- meridional advection-diffusion field (sediment model 3 without a supplied grid) ----------------
// The reference solves, per size bin, the stationary axisymmetric advection-diffusion of the sediment in
// the secondary (meridional) circulation of the stirred cell on a cell-centred (r, z) grid: upwind finite
// volumes with no-flux walls, red-black SOR, per-bin mass renormalisation every 20 iterations and at every
// convergence check, stopping at the first check (after at least min(1000, max) iterations) where the
// largest relative residual over all bins is within tolerance (CLARITAS/CLARITAS.py:4040-4215, driven by
// :6451-6725, one launch per half-sweep). Here one cooperative launch does all of it: a CTA per bin keeps
// its bin's plane in shared memory; the bins meet only at the checks (a bounded grid barrier) to agree on
// the largest residual. Every cell value, sum order and stopping iteration is the reference's.

// free-surface height and slope at radius r (:4046-4057)
__device__ void merid_surface(int FSM, double r, double ZMEAN, double R, double DH, double CORE, double* zs, double* hp) {
    double rr = fmin(fmax(r, 0.0), R), rr2 = rr * rr, R2 = R * R;
    *zs = ZMEAN; *hp = 0.0;
    if (!(DH > 0.0) || FSM == 0) return;
    if (FSM == 1) { *zs = ZMEAN + DH * (rr2 / R2 - 0.5); *hp = 2.0 * DH * rr / R2; return; }
    double a2 = CORE * CORE, Hinf = DH * (a2 + R2) / R2;
    double hbar = Hinf * (1.0 - (a2 / R2) * log1p(R2 / a2));
    *zs = ZMEAN - hbar + Hinf * rr2 / (a2 + rr2);
    *hp = 2.0 * Hinf * a2 * rr / ((a2 + rr2) * (a2 + rr2));
}
// secondary-circulation velocity from the streamfunction psi = -2U r^2 (1-r^2/R^2)^2 eta(1-eta) (:4059-4073)
__device__ void merid_velocity(double r, double z, double ZMIN, double ZMEAN, double R, int FSM, double DH, double CORE,
                               double UPEAK, double* ur, double* uz) {
    *ur = 0.0; *uz = 0.0;
    if (!(UPEAK > 0.0) || !(R > 0.0) || !(DH > 0.0) || (FSM == 2 && !(CORE > 0.0))) return;
    double rr = fmin(fmax(r, 0.0), R), R2 = R * R, rr2 = rr * rr, zs = ZMEAN, hp = 0.0;
    merid_surface(FSM, rr, ZMEAN, R, DH, CORE, &zs, &hp);
    double H = zs - ZMIN;
    if (!(H > 0.0)) return;
    double eta = (z - ZMIN) / H;
    if (eta < 0.0) eta = 0.0;
    if (eta > 1.0) eta = 1.0;
    double sq = rr2 / R2, f = eta * (1.0 - eta), fp = 1.0 - 2.0 * eta;
    double Apsi = 2.0 * UPEAK, om = 1.0 - sq;
    *ur = Apsi * rr * om * om * fp / H;
    *uz = -Apsi * (2.0 * om * (1.0 - 3.0 * sq) * f - rr * om * om * fp * eta * hp / H);
}
// radial slip interpolated from the per-bin table (:4075-4082)
__device__ double merid_slip(int p, double r, double R, const double* WR, int NRAD) {
    if (NRAD < 2 || !(R > 0.0)) return 0.0;
    double q = fmin(fmax(r / R, 0.0), 1.0) * (double)(NRAD - 1);
    int j = (int)floor(q);
    double t = q - (double)j;
    if (j >= NRAD - 1) { j = NRAD - 2; t = 1.0; }
    long long b = (long long)p * (long long)NRAD;
    return (1.0 - t) * WR[b + j] + t * WR[b + j + 1];
}
// a point inside the liquid (:4084-4089)
__device__ int merid_fluid(double r, double z, double ZMIN, double ZMEAN, double R, int FSM, double DH, double CORE) {
    if (z < ZMIN) return 0;
    double zs = ZMEAN, hp = 0.0;
    merid_surface(FSM, r, ZMEAN, R, DH, CORE, &zs, &hp);
    return z < zs;
}
// the finite-Re drift-diffusion field at a cell centre (sediment_local_scale with model 2, :1560-1593),
// which starts the iteration (:4100-4112)
__device__ double merid_initial(int FSM, int p, const double* SA, const double* SB, const double* SN, const double* RL,
                                int NRAD, float x, float z, float R, float ZMIN) {
    (void)FSM; (void)SA;
    double rr2 = (double)x * (double)x + 0.0 * 0.0;
    double R2 = (double)R * (double)R;
    if (rr2 > R2) rr2 = R2;
    double rr = sqrt(fmax(rr2, 0.0));
    double u = (R > 0.0) ? rr / (double)R * (double)(NRAD - 1) : 0.0;
    int j = (int)floor(u);
    if (j < 0) j = 0;
    if (j > NRAD - 2) j = NRAD - 2;
    double t = u - (double)j;
    long long base = (long long)p * (long long)NRAD;
    double radial_log = (1.0 - t) * RL[base + j] + t * RL[base + j + 1];
    if (radial_log > 0.0) radial_log = 0.0;
    double h = fmax((double)z - (double)ZMIN, 0.0);
    double logrel = radial_log - SB[p] * h;
    double ns = SN[p];
    if (!(ns > 0.0)) return 0.0;
    return exp(logrel) / ns;
}

__device__ __forceinline__ unsigned long long merid_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Barrier over the co-resident CTAs of a cooperative launch; gives up (error 91) after two seconds.
__device__ bool merid_grid_barrier(unsigned* count, unsigned* gen, unsigned nblocks, int* err) {
    __shared__ int ok_s;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok_s = 1;
        volatile unsigned* vgen = gen;
        const unsigned g = *vgen;
        __threadfence();
        if (atomicAdd(count, 1u) + 1u == nblocks) {
            *count = 0u;
            __threadfence();
            atomicAdd(gen, 1u);
        } else {
            const unsigned long long t0 = merid_ns();
            while (*vgen == g) {
                if (merid_ns() - t0 > 2000000000ull) { ok_s = 0; atomicCAS(err, 0, 91); break; }
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok_s != 0;
}

struct MeridArgs {
    int n, NR, NZ, NRAD, FSM, max_it, check_every;
    double R, ZMIN, ZMEAN, ZGRIDMAX, DH, CORE, UPEAK, Dt, OMEGA, TOL;
    const double *sedA, *sedB, *sed_norm, *radial_log, *wr, *ws;
    double* grid;       // [n][NR][NZ]
    double* coef;       // [n][5][NR*NZ]: AP, AE, AW, AN, AS
    double* grid_max;   // [n] largest value over the liquid cells
    double* residual;   // [2][n] residual of every bin at the last two checks
    unsigned* bar;      // [2] barrier count and generation (zero before the launch)
    int* err;           // first error code
    int* iterations;    // [1] iterations done (the reference's solver_iterations)
    double* max_residual;  // [1]
};

constexpr int kMeridThreads = 512;

__global__ void __launch_bounds__(kMeridThreads) meridional_solve_kernel(MeridArgs a) {
    extern __shared__ __align__(16) unsigned char msm[];
    const int NR = a.NR, NZ = a.NZ, plane = NR * NZ, p = blockIdx.x, tid = threadIdx.x;
    double* G = reinterpret_cast<double*>(msm);
    unsigned char* act = msm + (size_t)plane * 8;
    __shared__ double red[kMeridThreads / 32];
    __shared__ double scale_s;
    __shared__ int bad_s;
    const double dr = a.R / (double)NR, dz = (a.ZGRIDMAX - a.ZMIN) / (double)NZ;
    double* AP = a.coef + (size_t)p * 5 * plane;
    double* AE = AP + plane;
    double* AW = AE + plane;
    double* AN = AW + plane;
    double* AS = AN + plane;
    // liquid cells (:4091-4098) and the starting field (:4100-4112)
    for (int c = tid; c < plane; c += kMeridThreads) {
        const int i = c / NZ, k = c - i * NZ;
        const double r = ((double)i + 0.5) * dr, z = a.ZMIN + ((double)k + 0.5) * dz;
        act[c] = (unsigned char)(merid_fluid(r, z, a.ZMIN, a.ZMEAN, a.R, a.FSM, a.DH, a.CORE) ? 1 : 0);
    }
    __syncthreads();
    for (int c = tid; c < plane; c += kMeridThreads) {
        const int i = c / NZ, k = c - i * NZ;
        if (!act[c]) { G[c] = 0.0; continue; }
        const float x = (float)(((double)i + 0.5) * dr), z = (float)(a.ZMIN + ((double)k + 0.5) * dz);
        G[c] = merid_initial(a.FSM, p, a.sedA, a.sedB, a.sed_norm, a.radial_log, a.NRAD, x, z, (float)a.R,
                             (float)a.ZMIN);
    }
    // upwind finite-volume coefficients (:4114-4159)
    for (int c = tid; c < plane; c += kMeridThreads) {
        const int i = c / NZ, k = c - i * NZ;
        AP[c] = AE[c] = AW[c] = AN[c] = AS[c] = 0.0;
        if (!act[c]) continue;
        double rc = ((double)i + 0.5) * dr, zc = a.ZMIN + ((double)k + 0.5) * dz;
        double rw = (double)i * dr, re = (double)(i + 1) * dr;
        double Az = 0.5 * (re * re - rw * rw), ap = 0.0, ur = 0.0, uz = 0.0, V = 0.0, F = 0.0, diff = 0.0;
        if (i + 1 < NR && act[(i + 1) * NZ + k] && merid_fluid(re, zc, a.ZMIN, a.ZMEAN, a.R, a.FSM, a.DH, a.CORE)) {
            merid_velocity(re, zc, a.ZMIN, a.ZMEAN, a.R, a.FSM, a.DH, a.CORE, a.UPEAK, &ur, &uz);
            V = ur + merid_slip(p, re, a.R, a.wr, a.NRAD); F = V * re * dz; diff = a.Dt * re * dz / dr;
            AE[c] = diff + fmax(-F, 0.0); ap += diff + fmax(F, 0.0);
        }
        if (i > 0 && act[(i - 1) * NZ + k] && merid_fluid(rw, zc, a.ZMIN, a.ZMEAN, a.R, a.FSM, a.DH, a.CORE)) {
            merid_velocity(rw, zc, a.ZMIN, a.ZMEAN, a.R, a.FSM, a.DH, a.CORE, a.UPEAK, &ur, &uz);
            V = ur + merid_slip(p, rw, a.R, a.wr, a.NRAD); F = -V * rw * dz; diff = a.Dt * rw * dz / dr;
            AW[c] = diff + fmax(-F, 0.0); ap += diff + fmax(F, 0.0);
        }
        double zf = zc + 0.5 * dz;
        if (k + 1 < NZ && act[i * NZ + k + 1] && merid_fluid(rc, zf, a.ZMIN, a.ZMEAN, a.R, a.FSM, a.DH, a.CORE)) {
            merid_velocity(rc, zf, a.ZMIN, a.ZMEAN, a.R, a.FSM, a.DH, a.CORE, a.UPEAK, &ur, &uz);
            V = uz - a.ws[p]; F = V * Az; diff = a.Dt * Az / dz;
            AN[c] = diff + fmax(-F, 0.0); ap += diff + fmax(F, 0.0);
        }
        zf = zc - 0.5 * dz;
        if (k > 0 && act[i * NZ + k - 1] && merid_fluid(rc, zf, a.ZMIN, a.ZMEAN, a.R, a.FSM, a.DH, a.CORE)) {
            merid_velocity(rc, zf, a.ZMIN, a.ZMEAN, a.R, a.FSM, a.DH, a.CORE, a.UPEAK, &ur, &uz);
            V = uz - a.ws[p]; F = -V * Az; diff = a.Dt * Az / dz;
            AS[c] = diff + fmax(-F, 0.0); ap += diff + fmax(F, 0.0);
        }
        AP[c] = ap;
    }
    __syncthreads();
    // per-bin mass renormalisation (:4176-4187): the mass sum runs serially in the reference's order
    auto normalize = [&]() {
        if (tid == 0) {
            double mass = 0.0;
            for (int i = 0; i < NR; ++i) {
                double rw = (double)i * dr, re = (double)(i + 1) * dr, vol = 0.5 * (re * re - rw * rw) * dz;
                for (int k = 0; k < NZ; ++k) {
                    const int c = i * NZ + k;
                    if (act[c]) mass += G[c] * vol;
                }
            }
            double target = 0.5 * a.R * a.R * (a.ZMEAN - a.ZMIN);
            bad_s = (!(mass > 0.0) || !(target > 0.0) || !isfinite(mass)) ? 1 : 0;
            if (bad_s) atomicCAS(a.err, 0, 41);
            scale_s = bad_s ? 1.0 : target / mass;
        }
        __syncthreads();
        if (!bad_s) {
            const double sc = scale_s;
            for (int c = tid; c < plane; c += kMeridThreads)
                if (act[c]) G[c] *= sc;
        }
        __syncthreads();
    };
    // one colour of the red-black SOR sweep (:4161-4174)
    auto relax = [&](int parity) {
        for (int c = tid; c < plane; c += kMeridThreads) {
            const int i = c / NZ, k = c - i * NZ;
            if (!act[c] || ((i + k) & 1) != parity || !(AP[c] > 0.0)) continue;
            double num = 0.0;
            if (i + 1 < NR) num += AE[c] * G[(i + 1) * NZ + k];
            if (i > 0) num += AW[c] * G[(i - 1) * NZ + k];
            if (k + 1 < NZ) num += AN[c] * G[i * NZ + k + 1];
            if (k > 0) num += AS[c] * G[i * NZ + k - 1];
            double target = num / AP[c], old = G[c], nv = (1.0 - a.OMEGA) * old + a.OMEGA * target;
            if (!isfinite(nv) || nv < 1e-14) nv = 1e-14;
            G[c] = nv;
        }
        __syncthreads();
    };
    // largest relative residual of the bin (:4189-4197)
    auto residual = [&]() -> double {
        double mr = 0.0;
        for (int c = tid; c < plane; c += kMeridThreads) {
            const int i = c / NZ, k = c - i * NZ;
            if (!act[c] || !(AP[c] > 0.0)) continue;
            double num = 0.0;
            if (i + 1 < NR) num += AE[c] * G[(i + 1) * NZ + k];
            if (i > 0) num += AW[c] * G[(i - 1) * NZ + k];
            if (k + 1 < NZ) num += AN[c] * G[i * NZ + k + 1];
            if (k > 0) num += AS[c] * G[i * NZ + k - 1];
            double den = fmax(fabs(AP[c] * G[c]), 1e-30), q = fabs(AP[c] * G[c] - num) / den;
            if (q > mr) mr = q;
        }
        for (int o = 16; o > 0; o >>= 1) mr = fmax(mr, __shfl_xor_sync(0xffffffffu, mr, o));
        if ((tid & 31) == 0) red[tid >> 5] = mr;
        __syncthreads();
        double m = 0.0;
        for (int w = 0; w < kMeridThreads / 32; ++w) m = fmax(m, red[w]);
        __syncthreads();
        return m;
    };
    normalize();
    const int min_it = a.max_it < 1000 ? a.max_it : 1000;
    int done = 0, last_checked = 0, checks = 0;
    double worst = 0.0;
    bool stop = false;
    // the initial normalisation is checked before the first sweep (:6561-6575)
    if (!merid_grid_barrier(a.bar, a.bar + 1, gridDim.x, a.err)) stop = true;
    if (!stop && *(volatile int*)a.err) stop = true;
    for (int it = 1; it <= a.max_it && !stop; ++it) {
        relax(0);
        relax(1);
        if (it % 20 == 0) normalize();
        if (it % a.check_every == 0 || it == a.max_it) {
            normalize();
            const double r = residual();
            double* slot = a.residual + (size_t)(checks & 1) * a.n;
            if (tid == 0) slot[p] = r;
            if (!merid_grid_barrier(a.bar, a.bar + 1, gridDim.x, a.err)) break;
            worst = 0.0;
            for (int q = 0; q < a.n; ++q) worst = fmax(worst, ((volatile double*)slot)[q]);
            last_checked = it;
            ++checks;
            if (*(volatile int*)a.err) break;
            if (it >= min_it && worst <= a.TOL) { done = it; break; }
        }
    }
    if (done == 0) done = last_checked ? last_checked : a.max_it;
    if (p == 0 && tid == 0) { *a.iterations = done; *a.max_residual = worst; }
    // extend each column above the free surface with its highest liquid value (:4199-4205)
    for (int i = tid; i < NR; i += kMeridThreads) {
        int top = -1;
        for (int k = NZ - 1; k >= 0; --k)
            if (act[i * NZ + k]) { top = k; break; }
        if (top < 0) { for (int k = 0; k < NZ; ++k) G[i * NZ + k] = 1.0; continue; }
        const double q = G[i * NZ + top];
        for (int k = top + 1; k < NZ; ++k) G[i * NZ + k] = q;
    }
    __syncthreads();
    double mx = 0.0;
    for (int c = tid; c < plane; c += kMeridThreads) {
        a.grid[(size_t)p * plane + c] = G[c];
        if (act[c] && G[c] > mx) mx = G[c];
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((tid & 31) == 0) red[tid >> 5] = mx;
    __syncthreads();
    if (tid == 0) {
        double m = 0.0;
        for (int w = 0; w < kMeridThreads / 32; ++w) m = fmax(m, red[w]);
        a.grid_max[p] = m;  // the majorant kernel takes 1 where this is not positive (:4207-4209)
    }
}

size_t meridional_coef_doubles(int n, int nr, int nz) { return (size_t)n * 5 * nr * nz; }

cudaError_t enqueue_meridional_solve(ParticleBuffers& pb, const clr_scene_params& sp, const clr_sediment_spec& ss,
                                     cudaStream_t st) {
    MeridArgs a;
    a.n = pb.n; a.NR = pb.grid_nr; a.NZ = pb.grid_nz; a.NRAD = pb.n_radial; a.FSM = sp.free_surface_model;
    a.max_it = ss.solver_max_iterations; a.check_every = ss.solver_check_interval;
    a.R = ss.rin; a.ZMIN = ss.zmin; a.ZMEAN = ss.zmean; a.ZGRIDMAX = ss.grid_zmax; a.DH = ss.vortex_delta_h;
    a.CORE = ss.vortex_core_radius; a.UPEAK = ss.meridional_peak_speed; a.Dt = ss.eddy_diffusivity;
    a.OMEGA = ss.solver_sor; a.TOL = ss.solver_tolerance;
    a.sedA = pb.sedA; a.sedB = pb.sedB; a.sed_norm = pb.sed_norm; a.radial_log = pb.sed_radial_log; a.wr = pb.sed_wr;
    a.ws = pb.sed_ws; a.grid = pb.sed_grid; a.coef = pb.merid_coef; a.grid_max = pb.grid_max;
    a.residual = pb.merid_residual; a.bar = pb.merid_bar; a.err = pb.err; a.iterations = pb.merid_stats;
    a.max_residual = reinterpret_cast<double*>(pb.merid_residual + 2 * (size_t)pb.n);
    const size_t smem = (size_t)a.NR * a.NZ * 9;
    cudaError_t e = cudaFuncSetAttribute(meridional_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(pb.merid_bar, 0, 2 * sizeof(unsigned), st)) != cudaSuccess) return e;
    void* args[] = {&a};
    return cudaLaunchCooperativeKernel((const void*)meridional_solve_kernel, dim3(a.n), dim3(kMeridThreads), args,
                                       smem, st);
}

// Upper bound of the orders the Mie kernel needs for n bins: the largest nmx = max(nstop, |m x|) + 128 of
// the bins (:3506-3512), recomputed on the host from the same inputs with a few orders of slack for
// libm differences in cbrt and hypot, and never above CLR_MIE_MAX_ORDER (bins past that limit fail in
// the kernel with the reference's error code 1 before using shared memory).
int mie_order_bound(const double* d, const double* nr, const double* k, int n, double n_medium, double wavelength) {
    int cap = 1;
    for (int i = 0; i < n; ++i) {
        const double x = PD_PI * n_medium * d[i] / wavelength;
        if (!(x > 0.0) || !(n_medium > 0.0)) continue;
        const double mz = std::hypot(nr[i] / n_medium * x, k[i] / n_medium * x);
        const double nstop = x + 4.0 * std::cbrt(x) + 2.0;
        const double nmx = std::fmax(nstop, mz) + 128.0 + 8.0;
        cap = nmx >= (double)CLR_MIE_MAX_ORDER ? CLR_MIE_MAX_ORDER : std::max(cap, (int)nmx + 1);
    }
    return std::min(cap, (int)CLR_MIE_MAX_ORDER);
}

static cudaError_t set_table_attributes() {
    cudaError_t e = cudaFuncSetAttribute(mie_coefficients_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kMieSmem);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(phase_pdf_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPdfSmem);
}

// Mie coefficients and efficiencies of n bins, then (hybrid event models) the theta grid and the phase
// pdf and CDF, else the two-point placeholder tables. `b.ab` holds n * order_cap a_n/b_n pairs and
// `b.pdf` n * nt values. The error word is not reset here.
cudaError_t enqueue_mie_tables(const double* d, const double* nr, const double* k, int n, double n_medium,
                               double wavelength, int nt, bool hybrid, int order_cap, const MiePhaseBuffers& b,
                               cudaStream_t st, bool fast_pdf) {
    cudaError_t e = set_table_attributes();
    if (e != cudaSuccess) return e;
    mie_coefficients_kernel<<<n, 32, mie_smem_bytes(order_cap), st>>>(d, nr, k, n_medium, wavelength, n, order_cap,
                                                                      b.ab, b.nstop, b.x, b.qext, b.qsca, b.qabs,
                                                                      b.qback, b.g, b.albedo, b.err);
    if (hybrid) {
        theta_grid_kernel<<<(nt + 127) / 128, 128, 0, st>>>(b.theta, b.theta_f, nt);
        if (fast_pdf) {
            dim3 grid(((nt + 1) / 2 + 127) / 128, (n + kPdfFastGroup - 1) / kPdfFastGroup);
            phase_pdf_fast_kernel<<<grid, 128, 0, st>>>(b.theta, nt, n, order_cap, b.nstop, b.ab, b.pdf);
        } else {
            dim3 grid((nt + 127) / 128, (n + PDF_GROUP - 1) / PDF_GROUP);
            phase_pdf_kernel<<<grid, 128, pdf_smem_bytes(order_cap), st>>>(b.theta, nt, n, order_cap, b.nstop,
                                                                            b.ab, b.pdf);
        }
        phase_cdf_kernel<<<n, 32, 0, st>>>(b.theta, b.pdf, nt, n, b.cdf, b.cdf_f, b.err);
    } else {
        dummy_phase_kernel<<<(n + 127) / 128, 128, 0, st>>>(b.theta, b.theta_f, b.cdf, b.cdf_f, n);
    }
    if (b.guide) {
        const long long cells = (long long)n * (kPhaseGuide + 1);
        phase_guide_kernel<<<(unsigned)((cells + 255) / 256), 256, 0, st>>>(b.cdf_f, hybrid ? nt : 2, n, b.guide);
    }
    return cudaGetLastError();
}

// Mie efficiencies, asymmetry, theta grid and phase CDF of n bins into buffers the caller supplies
// (the first steps of enqueue_particle_precompute, with no buffer of its own). Used by the
// allocation-free entry point.
cudaError_t enqueue_mie_phase(const double* d, const double* nr, const double* k, int n, double n_medium,
                              double wavelength, int nt, const MiePhaseBuffers& b, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(b.err, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    return enqueue_mie_tables(d, nr, k, n, n_medium, wavelength, nt, true, CLR_MIE_MAX_ORDER, b, st);
}

static TransportJob transport_job_of(ParticleBuffers& pb, const clr_scene_params& sp, const clr_particle_spec& ps) {
    TransportJob j;
    j.n = pb.n; j.weight_mode = ps.weight_mode; j.em = sp.event_model;
    j.d = pb.d; j.w_in = pb.w; j.qext = pb.qext; j.qsca = pb.qsca; j.k_imag = pb.kidx; j.n_real = pb.nidx;
    j.concentration = ps.concentration_kg_m3; j.density = ps.density_kg_m3; j.wave_scale = ps.hybrid_wave_scale;
    j.n_medium = ps.n_medium; j.wavelength = ps.wavelength_m; j.wave_rms = ps.wave_rms_height_m;
    j.w = pb.w; j.radius = pb.radius; j.nden = pb.nden; j.mug = pb.mug; j.mus = pb.mus; j.mue = pb.mue;
    j.muw = pb.muw; j.muev = pb.muev; j.gcdf = pb.gcdf; j.wcdf = pb.wcdf; j.pcdf = pb.pcdf; j.muscal = pb.muscal;
    j.trace_geom = pb.trace_geom; j.trace_wave = pb.trace_wave; j.gcdf_f = pb.gcdf_f; j.wcdf_f = pb.wcdf_f;
    j.pn_f = pb.pn_f; j.pk_f = pb.pk_f; j.prad_f = pb.prad_f; j.error_flag = pb.err;
    return j;
}

static SedArgs sed_args_of(const ParticleBuffers& pb, const clr_scene_params& sp, const clr_sediment_spec& ss) {
    SedArgs a;
    a.n = pb.n; a.TM = sp.sediment_model; a.FSM = sp.free_surface_model; a.NQ = ss.n_quad; a.NRAD = ss.n_radial;
    a.rho_p = ss.particle_density; a.rho_w = ss.water_density; a.mu = ss.water_viscosity; a.grav = ss.gravity;
    // FP64 geometry as the reference passes it to its sediment kernels (the host fills it from the scene's
    // FP32 values when the caller leaves it zero)
    a.Dt = ss.eddy_diffusivity; a.R = ss.rin; a.ZMIN = ss.zmin; a.ZMEAN = ss.zmean;
    a.DH = ss.vortex_delta_h; a.CORE = ss.vortex_core_radius;
    (void)sp;
    return a;
}

static MajorantJob majorant_job_of(ParticleBuffers& pb, const SedArgs& a) {
    MajorantJob j;
    j.a = a; j.trace_geom = pb.trace_geom; j.trace_wave = pb.trace_wave; j.grid_max = a.TM == 3 ? pb.grid_max : nullptr;
    j.sed_A = pb.sedA; j.sed_norm = pb.sed_norm; j.sed_max = pb.sed_max; j.major = pb.sed_major; j.error_flag = pb.err;
    return j;
}

// Sediment bin coefficients (and the finite-Re slip table, the grid maxima) of one scenario.
static void enqueue_sediment_bins(ParticleBuffers& pb, const SedArgs& a, cudaStream_t st) {
    if (a.TM == 2 || a.TM == 3) {
        dim3 g((a.NRAD + 127) / 128, a.n);
        sediment_slip_kernel<<<g, 128, 0, st>>>(a, pb.d, pb.sed_wr);
    }
    sediment_bin_kernel<<<a.n, 32, 0, st>>>(a, pb.d, pb.sed_wr, pb.sedA, pb.sedB, pb.sed_norm, pb.sed_max,
                                            pb.sed_radial_log, pb.sed_terms, pb.sed_ws, pb.err);
    if (a.TM == 3 && !pb.merid_coef)  // a supplied grid: its largest value per bin (the solver gives its own)
        sediment_grid_max_kernel<<<a.n, 256, 0, st>>>(pb.sed_grid, (long long)pb.grid_nr * pb.grid_nz, pb.grid_max);
}

static cudaError_t enqueue_node_tables(ParticleBuffers& pb, cudaStream_t st) {
    if (!pb.node_tables) return cudaSuccess;
    const int plane = pb.grid_nr * pb.grid_nz;
    cudaError_t e = cudaMemsetAsync(pb.node_major, 0, sizeof(float), st);
    if (e != cudaSuccess) return e;
    sediment_node_kernel<<<(2 * plane + 127) / 128, 128, 0, st>>>(pb.sed_grid, pb.trace_geom, pb.trace_wave, pb.n,
                                                                  plane, pb.node_mu, pb.node_alias,
                                                                  reinterpret_cast<unsigned int*>(pb.node_major));
    return cudaSuccess;
}

// The scene-dependent rest of the precompute of one scenario, after its Mie tables: PSD normalisation
// and rates, sediment coefficients, majorants and node tables.
cudaError_t enqueue_scene_rates(ParticleBuffers& pb, const clr_scene_params& sp, const clr_particle_spec& ps,
                                const clr_sediment_spec& ss, cudaStream_t st) {
    transport_kernel<<<1, 1, 0, st>>>(transport_job_of(pb, sp, ps));
    const SedArgs a = sed_args_of(pb, sp, ss);
    enqueue_sediment_bins(pb, a, st);
    if (pb.merid_coef) {
        cudaError_t e = enqueue_meridional_solve(pb, sp, ss, st);
        if (e != cudaSuccess) return e;
    }
    sediment_majorant_kernel<<<1, 1, 0, st>>>(majorant_job_of(pb, a));
    cudaError_t e = enqueue_node_tables(pb, st);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

size_t scene_rates_batch_scratch(int n) { return (size_t)n * (sizeof(TransportJob) + sizeof(MajorantJob)) + 256; }

// The same for n scenarios: the one-thread rate and majorant kernels of all scenarios run as one launch
// each (a thread per scenario); the sediment bins and node tables stay per scenario. `d_scratch` holds
// scene_rates_batch_scratch(n) bytes of device memory for the job descriptions.
cudaError_t enqueue_scene_rates_batch(ParticleBuffers* const* pbs, const clr_scene_params* sps,
                                      const clr_particle_spec* pss, const clr_sediment_spec* sss, int n,
                                      void* d_scratch, cudaStream_t st) {
    std::vector<TransportJob> tj(n);
    std::vector<MajorantJob> mj(n);
    std::vector<SedArgs> sa(n);
    for (int i = 0; i < n; ++i) {
        tj[i] = transport_job_of(*pbs[i], sps[i], pss[i]);
        sa[i] = sed_args_of(*pbs[i], sps[i], sss[i]);
        mj[i] = majorant_job_of(*pbs[i], sa[i]);
    }
    TransportJob* d_tj = static_cast<TransportJob*>(d_scratch);
    MajorantJob* d_mj = reinterpret_cast<MajorantJob*>(
        (reinterpret_cast<uintptr_t>(d_tj + n) + 255) & ~(uintptr_t)255);
    // pageable sources: the copies are staged before the calls return
    cudaError_t e = cudaMemcpyAsync(d_tj, tj.data(), n * sizeof(TransportJob), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    e = cudaMemcpyAsync(d_mj, mj.data(), n * sizeof(MajorantJob), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    transport_batch_kernel<<<(n + 63) / 64, 64, 0, st>>>(d_tj, n);
    for (int i = 0; i < n; ++i) enqueue_sediment_bins(*pbs[i], sa[i], st);
    for (int i = 0; i < n; ++i)
        if (pbs[i]->merid_coef && (e = enqueue_meridional_solve(*pbs[i], sps[i], sss[i], st)) != cudaSuccess) return e;
    sediment_majorant_batch_kernel<<<(n + 63) / 64, 64, 0, st>>>(d_mj, n);
    for (int i = 0; i < n; ++i)
        if ((e = enqueue_node_tables(*pbs[i], st)) != cudaSuccess) return e;
    return cudaGetLastError();
}

cudaError_t enqueue_particle_precompute(ParticleBuffers& pb, const clr_scene_params& sp, const clr_particle_spec& ps,
                                        const clr_sediment_spec& ss, double* ab_scratch, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(pb.err, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    MiePhaseBuffers b;
    b.ab = ab_scratch ? ab_scratch : pb.ab;
    b.nstop = pb.nstop; b.x = pb.x; b.qext = pb.qext; b.qsca = pb.qsca; b.qabs = pb.qabs; b.qback = pb.qback;
    b.g = pb.g; b.albedo = pb.albedo; b.theta = pb.theta; b.theta_f = pb.theta_f; b.pdf = pb.pdf;
    b.cdf = pb.phase_cdf; b.cdf_f = pb.phase_cdf_f; b.guide = pb.phase_guide; b.err = pb.err;
    const int em = sp.event_model;
    e = enqueue_mie_tables(pb.d, pb.nidx, pb.kidx, pb.n, ps.n_medium, ps.wavelength_m, pb.nt,
                           em == 3 || em == 4 || em == 5, CLR_MIE_MAX_ORDER, b, st,
                           ps.table_arithmetic == CLR_TABLES_FAST);
    if (e != cudaSuccess) return e;
    return enqueue_scene_rates(pb, sp, ps, ss, st);
}

}  // namespace clr
