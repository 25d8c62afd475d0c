// Photon history as a resumable state machine.
//
// The reference traces each ray start-to-finish in one thread (trace_kernel,
// CLARITAS/CLARITAS.py:4551-5104) and scores it in a second kernel
// (score_detectors_kernel :4378-4436). Here a history is split into
// resumable steps -- the launch segment (source, collimator, acrylic entry,
// :4650-4732) and one water free-flight step (one iteration of :4734-5066) --
// so a persistent warp can hand a finished lane a fresh photon immediately.
// Within each step the arithmetic, random-draw order and branch structure are
// the reference's, so per-ray integer outcomes are reproduced exactly in the
// xorshift parity mode.
#pragma once
#include "physics_b.cuh"
#include "device_scene.cuh"

namespace clr {
namespace {  // header-only device code: internal linkage in every translation unit

// Phases of a history. SOURCE (FP32 sampling up to collimator acceptance) rejects most photons;
// ENTRY (outer-wall Fresnel, acrylic solid, headspace) and WATER are the FP64-heavy phases.
enum : int { PHASE_SOURCE = 0, PHASE_ENTRY = 1, PHASE_WATER = 2 };

struct Ray {
    float x, y, z, vx, vy, vz, wp, ap, w;
    int phase, step, st, pf, pfs;
    int ic, gic, wic, wcoh, wmorph, cir, cor, ctir, tr, ttir, bir, bor, btir, sbi, sbr, entered;
    o_pcount pc;
    int steps, nulls;
};

// Small per-history counters that the reference keeps in registers; summed into tallies at the end.
__device__ __forceinline__ void ray_reset(Ray& r) {
    r.x = r.y = r.z = 0.f; r.vx = 0.f; r.vy = 1.f; r.vz = 0.f; r.wp = 0.f; r.ap = 0.f; r.w = 1.f;
    r.phase = PHASE_SOURCE; r.step = 0; r.st = 0; r.pf = 0; r.pfs = 0;
    r.ic = r.gic = r.wic = r.wcoh = r.wmorph = 0;
    r.cir = r.cor = r.ctir = r.tr = r.ttir = r.bir = r.bor = r.btir = r.sbi = r.sbr = r.entered = 0;
    r.pc.reflections = r.pc.entry_reflections = r.pc.internal_reflections = r.pc.absorptions = 0;
    r.steps = r.nulls = 0;
}

// per-warp shared tally region (64-bit counters; flushed to the owning scenario's DevTally)
typedef TallyCore WarpTally;

// offsets inside WarpTally/DevTally counter space (in units of unsigned long long after hw)
#define CLR_OFF_HW(k, j) ((k) * CLR_N_DETECTORS + (j))
#define CLR_OFF_STATUS (10 * CLR_N_DETECTORS + 8 * CLR_N_DETECTORS)
#define CLR_OFF_FAIL (CLR_OFF_STATUS + CLR_N_STATUS)
#define CLR_OFF_EV (CLR_OFF_FAIL + CLR_N_FAILURE_CODES)
#define CLR_OFF_CS (CLR_OFF_EV + CLR_N_EVENT_COUNTERS)
#define CLR_OFF_DONE (CLR_OFF_CS + CLR_N_CONDITIONAL_STATS)
#define CLR_OFF_ES (CLR_OFF_DONE + 1)
#define CLR_OFF_RF (CLR_OFF_ES + 16)
#define CLR_OFF_SUB (CLR_OFF_RF + 16)
#define CLR_OFF_ICLO (CLR_OFF_SUB + CLR_N_SUBCODES)

// ---------------- conditional closure (:4479-4536) ----------------
struct Hist {
    float x, y, z, vx, vy, vz, path;
    o_pcount pc;
    int status, channel, macro, micro, failure, subcode;
};

// Loop state of a closure, so that its trials can run in bounded pieces (a closure can take 16384).
struct CondState {
    int started;  // setup (argument checks, the absorbed/scattered target draw) done
    int trial;    // next trial
    int target;   // pre-drawn target outcome: 1 absorbed, 0 scattered
};
__device__ __forceinline__ CondState cond_start() {
    CondState c = {0, 0, 0};
    return c;
}

// Inputs of a closure's candidate histories: the same for every trial of one closure.
struct ClosureIn {
    const float* cdf;
    const float* theta;
    const int* guide;
    double wave;
    float nm, nr, ki, wl, rough, radius, aspect, kappa, coherent;
    float x, y, z, vx, vy, vz, rin, zmin, zmean, delta, core;
    int pidx, orientation, max_bounces, nt, surface;
};

// One candidate history of a closure (one iteration of the trial loop, :4505-4533). Returns -2 when the
// sampled sphere does not fit in the water, -1 when the outcome is not the target, and 1 when the trial
// ends the closure with *h: the target outcome, or a failure when h->status is neither 1 nor 2.
template <class S>
__device__ __forceinline__ int closure_trial(S* s, const ClosureIn& c, int target_absorbed, Hist* h) {
    const float x = c.x, y = c.y, z = c.z, vx = c.vx, vy = c.vy, vz = c.vz, radius = c.radius;
    memset(h, 0, sizeof *h);
    h->x = x; h->y = y; h->z = z; h->vx = vx; h->vy = vy; h->vz = vz;
    h->channel = (uniform53(s) < c.wave) ? ((c.coherent >= 1.0f || uniform53(s) < c.coherent) ? 1 : 2) : 0;
    if (h->channel == 1) {
        o_mie_direction(s, c.cdf, c.theta, c.nt, c.pidx, &h->vx, &h->vy, &h->vz, c.guide);
        h->status = 1;
    } else if (h->channel == 2) {
        float fr = sqrtf(x * x + y * y), fx = 1, fy = 0;
        if (fr > 1e-12f) { fx = -y / fr; fy = x / fr; }
        h->status = o_spheroid_event(s, c.nm, c.nr, c.ki, c.wl, c.rough, radius, c.aspect, c.orientation, c.kappa, fx,
                                     fy, 0, c.max_bounces, &h->vx, &h->vy, &h->vz, &h->path, &h->pc, &h->failure,
                                     &h->subcode, &h->macro, &h->micro);
    } else {
        float rho, phi, gx, gy, gz;
        o_sphere_geometry(s, radius, x, y, z, vx, vy, vz, &rho, &phi, &gx, &gy, &gz);
        if constexpr (kCounterStream<S>) {
            const float fcx = x - radius * gx, fcy = y - radius * gy, fcz = z - radius * gz;
            if (!f_sphere_accessible(fcx, fcy, fcz, radius, c.rin, c.zmin, c.zmean, c.surface, c.delta, c.core))
                return -2;
            h->status = f_sphere_sampled(s, c.nm, c.nr, c.ki, c.wl, c.rough, radius, c.max_bounces, gx, gy, gz, fcx,
                                         fcy, fcz, &h->x, &h->y, &h->z, &h->vx, &h->vy, &h->vz, &h->path, &h->pc,
                                         &h->failure, &h->subcode, &h->macro, &h->micro);
        } else {
            double dcx = (double)x - (double)radius * gx, dcy = (double)y - (double)radius * gy,
                   dcz = (double)z - (double)radius * gz;
            if (!o_sphere_accessible(dcx, dcy, dcz, radius, c.rin, c.zmin, c.zmean, c.surface, c.delta, c.core))
                return -2;
            h->status = o_sphere_sampled(s, c.nm, c.nr, c.ki, c.wl, c.rough, radius, c.max_bounces, gx, gy, gz, dcx,
                                         dcy, dcz, &h->x, &h->y, &h->z, &h->vx, &h->vy, &h->vz, &h->path, &h->pc,
                                         &h->failure, &h->subcode, &h->macro, &h->micro);
        }
    }
    if (h->status != 1 && h->status != 2) return 1;
    if ((h->status == 2) != target_absorbed) return -1;
    return 1;
}

// Setup of a closure (argument checks and the absorbed/scattered target draw, :4491-4504). Returns 1 with
// *out set when the closure ends here, else 0 with cs->target set.
template <class S>
__device__ __forceinline__ int closure_setup(S* s, Hist* out, double qs, double qe, float ki, int max_trials,
                                             unsigned long long* stats, CondState* cs, float* wmul) {
    Hist h;
    memset(&h, 0, sizeof h);
    h.failure = OP_OTHER; h.subcode = 9002;
    double tol = 1e-10 * fmax(1.0, fmax(fabs(qs), fabs(qe)));
    double albedo = (ki == 0.0f && fabs(qe - qs) <= tol) ? 1.0 : fmin(fmax(qs / qe, 0.0), 1.0);
    if (max_trials == 0) { h.subcode = 9001; ++stats[9]; *out = h; return 1; }
    if (!isfinite(qs) || !isfinite(qe) || qe <= 0.0 || qs < -tol || qs > qe + tol || max_trials < 1) { ++stats[8]; *out = h; return 1; }
    double pabs = (ki == 0.0f && fabs(qe - qs) <= tol) ? 0.0 : fmin(fmax((qe - qs) / qe, 0.0), 1.0);
    const double MINP = 2.3283064365386962890625e-10;
    if ((ki > 0.0f && (pabs <= 0.0 || albedo >= 1.0)) || (albedo > 0.0 && albedo < MINP) || (pabs > 0.0 && pabs < MINP)) {
        h.subcode = 9003; ++stats[8]; *out = h; return 1;
    }
    if (wmul && albedo > 0.0) {
        // implicit capture (weighted runs): the photon always scatters and carries the survival
        // probability instead of drawing the absorbed/scattered outcome
        *wmul *= (float)albedo;
        cs->target = 0;
    } else {
        cs->target = (albedo < 1.0 && uniform53(s) >= albedo);
    }
    cs->started = 1;
    cs->trial = 0;
    return 0;
}

// Counter word 2 of the substream of closure trial t (counter-based stream): a tag bit, the photon's
// event number (17 bits) and t (14 bits; trials per closure are at most 16384, checked per run).
constexpr int kClosureTrialBits = 14;
__device__ __forceinline__ uint32_t closure_trial_tag(int ic) {
    return 0x80000000u | (((uint32_t)ic & 0x1FFFFu) << kClosureTrialBits);
}

__device__ __forceinline__ Hist closure_exhausted(unsigned long long* stats) {
    Hist h;
    memset(&h, 0, sizeof h);
    h.failure = OP_OTHER; h.subcode = 9001;
    ++stats[9];
    return h;
}

// Runs the closure from *cs for at most `budget` trials (0: to its end). Returns 1 with *out set when
// the closure finished, 0 when the budget ran out first (state in *cs).
template <class S>
__device__ __forceinline__ int conditional_body(
    S* s, Hist* out, int pidx, double qs, double qe, float nm, float nr, float ki, float wl, float rough,
    float radius, float aspect, int orientation, float kappa, int max_bounces, float coherent, const float* cdf,
    const float* theta, const int* guide, int nt, float x, float y, float z, float vx, float vy, float vz, float rin,
    float zmin, float zmean, int surface, float delta, float core, int max_trials, unsigned long long* stats, CondState* cs,
    int budget, float* wmul, uint32_t trial_tag) {
    if (!cs->started && closure_setup(s, out, qs, qe, ki, max_trials, stats, cs, wmul)) return 1;
    const int target_absorbed = cs->target;
    ClosureIn c;
    c.cdf = cdf; c.theta = theta; c.guide = guide; c.wave = qs > 0.0 ? fmax(qs - 1.0, 0.0) / qs : 0.0;
    c.nm = nm; c.nr = nr; c.ki = ki; c.wl = wl; c.rough = rough; c.radius = radius; c.aspect = aspect;
    c.kappa = kappa; c.coherent = coherent;
    c.x = x; c.y = y; c.z = z; c.vx = vx; c.vy = vy; c.vz = vz; c.rin = rin; c.zmin = zmin; c.zmean = zmean;
    c.delta = delta; c.core = core;
    c.pidx = pidx; c.orientation = orientation; c.max_bounces = max_bounces; c.nt = nt; c.surface = surface;
    const int end = (budget > 0 && max_trials - cs->trial > budget) ? cs->trial + budget : max_trials;
    Hist h;
    for (int trial = cs->trial; trial < end; ++trial) {
        ++stats[0];
        int t;
        if constexpr (kCounterStream<S>) {
            // trial `trial` on its own substream, as the warp-cooperative closure draws it: the result of a
            // photon does not depend on which of the two runs its closure
            S ts = *s;
            ts.c2 = trial_tag | (uint32_t)trial;
            ts.draw = 0u;
            ts.idx = 4;
            t = closure_trial(&ts, c, target_absorbed, &h);
        } else {
            t = closure_trial(s, c, target_absorbed, &h);
        }
        if (t == -2) { ++stats[2]; continue; }
        if (t == -1) { ++stats[1]; continue; }
        if (h.status != 1 && h.status != 2) { ++stats[8]; *out = h; return 1; }
        ++stats[3 + h.channel];
        ++stats[h.status == 2 ? 6 : 7];
        *out = h;
        return 1;
    }
    if (end < max_trials) { cs->trial = end; return 0; }
    *out = closure_exhausted(stats);
    return 1;
}

// The encounter's trial counters are thread-local and merged atomically once per call, as the
// reference's conditional_particle_interaction_accumulate does once per encounter (:4540-4549);
// the sums are the same.
template <class S>
__device__ __noinline__ int conditional_interaction(
    S* s, Hist* out, int pidx, double qs, double qe, float nm, float nr, float ki, float wl, float rough,
    float radius, float aspect, int orientation, float kappa, int max_bounces, float coherent, const float* cdf,
    const float* theta, const int* guide, int nt, float x, float y, float z, float vx, float vy, float vz, float rin,
    float zmin, float zmean, int surface, float delta, float core, int max_trials, unsigned long long* gstats,
    CondState* cs, int budget, float* wmul, uint32_t trial_tag) {
    unsigned long long stats[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    const int done = conditional_body(s, out, pidx, qs, qe, nm, nr, ki, wl, rough, radius, aspect, orientation, kappa,
                                      max_bounces, coherent, cdf, theta, guide, nt, x, y, z, vx, vy, vz, rin, zmin,
                                      zmean, surface, delta, core, max_trials, stats, cs, budget, wmul, trial_tag);
#pragma unroll
    for (int i = 0; i < 10; ++i)
        if (stats[i]) atomicAdd(gstats + i, stats[i]);
    return done;
}

// Mie two-moment post-outcome angular map (:4459-4476)
__device__ __noinline__ void moment_constraint(float vinx, float viny, float vinz, float* vx, float* vy, float* vz,
                                               float A, float B) {
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

__device__ __forceinline__ o_cell make_cell(const clr_scene_params& P) {
    o_cell C = {P.n_water, P.n_acrylic, P.n_air, P.bottom_external_n, P.rin, P.rout, P.zmin,
                P.zmin - P.bottom_disc_thickness, P.zmean, P.zwall_top, P.free_surface_model, P.vortex_delta_h,
                P.vortex_core_radius};
    return C;
}
__device__ __forceinline__ o_field make_field(const DevScene& D) {
    o_field F = {D.P.sediment_model, D.P.free_surface_model, D.n_bins, D.n_radial, D.grid_nr, D.grid_nz,
                 D.sedA, D.sedB, D.sed_norm, D.sed_radial_log, D.sed_grid, D.grid_zmax, D.P.rin, D.P.zmin,
                 D.P.vortex_core_radius};
    return F;
}

// Add the acrylic/headspace bounce counters of a sub-path to the ray.
__device__ __forceinline__ void add_bounces(Ray& r, const o_bcount& b) {
    r.cir += b.cir; r.cor += b.cor; r.ctir += b.ctir; r.tr += b.tr; r.ttir += b.ttir;
    r.bir += b.bir; r.bor += b.bor; r.btir += b.btir;
}

// ---------------- source segment: emission and collimator (:4650-4711) ----------------
// Returns true when the history ended (rejected, r.st = 3); otherwise the ray waits in PHASE_ENTRY.
template <class S>
__device__ __forceinline__ bool source_segment(const DevScene& D, Ray& r, S* src) {
    const clr_scene_params& P = D.P;
    float x, y, z, vx = 0.0f, vy = 1.0f, vz = 0.0f;
    if (P.source_kind == CLR_SOURCE_COLLIMATED_DISC) {
        // New source (no reference counterpart): a uniform disc of radius disc_radius centred on the
        // 180-degree axis at height disc_height, travelling along +y from just inside the sensor-ring radius.
        float u1 = uniform(src), u2 = uniform(src);
        float rr = P.disc_radius * sqrtf(u1);
        float ph = 2.0f * CLR_PI_F * u2;
        x = rr * cosf(ph);
        z = P.disc_height + rr * sinf(ph);
        y = -P.ring_in;
    } else {
        float u1 = fmaxf(uniform(src), 1e-12f), u2 = uniform(src);
        float mag = sqrtf(-2.0f * logf(u1));
        x = P.beam_sigma * mag * cosf(2.0f * CLR_PI_F * u2);
        z = P.beam_sigma * mag * sinf(2.0f * CLR_PI_F * u2);
        y = -P.source_r;
        float polar, az;
        if (P.source_angular_model == 0) {
            polar = o_beta(src, P.alpha1, P.alpha2) * (CLR_PI_F / 2.0f);
            az = 2.0f * CLR_PI_F * uniform(src);
            float sp = sinf(polar);
            vx = sp * cosf(az); vy = cosf(polar); vz = sp * sinf(az);
        } else if (P.source_angular_model == 1) {
            polar = o_beta_radiance_polar(src, P.alpha1, P.alpha2);
            az = 2.0f * CLR_PI_F * uniform(src);
            float sp = sinf(polar);
            vx = sp * cosf(az); vy = cosf(polar); vz = sp * sinf(az);
        } else {
            float h = o_beta(src, P.alpha1, P.alpha2) * (CLR_PI_F / 2.0f);
            if (uniform(src) < 0.5f) h = -h;
            vx = sinf(h); vy = cosf(h); vz = 0.0f;
        }
        o_normalize(&vx, &vy, &vz);
        if (vy <= 1e-12f) { r.st = 3; return true; }
        if (P.source_bore_model == 0) {
            if (x * x + z * z > P.counterbore_r * P.counterbore_r) { r.st = 3; return true; }
            float t = (-P.throat_out - y) / vy;
            if (t < -CLR_EPS_F) { r.st = 3; return true; }
            if (t < 0.0f) t = 0.0f;
            float xt = x + t * vx, zt = z + t * vz;
            if (xt * xt + zt * zt > P.throat_r * P.throat_r) { r.st = 3; return true; }
            t = (-P.ring_in - y) / vy;
            if (t <= 0.0f) { r.st = 3; return true; }
            x += t * vx; y += t * vy; z += t * vz;
            if (x * x + z * z > P.throat_r * P.throat_r) { r.st = 3; return true; }
        } else {
            if (!o_source_collimator(src, P.source_bore_model, P.n_air, P.bore_n, P.max_bore_bounces, P.ring_in,
                                     P.throat_out, P.source_r, P.throat_r, P.counterbore_r, &x, &y, &z, &vx, &vy, &vz,
                                     &r.sbi, &r.sbr)) { r.st = 3; return true; }
        }
    }
    r.x = x; r.y = y; r.z = z; r.vx = vx; r.vy = vy; r.vz = vz;
    r.phase = PHASE_ENTRY;
    return false;
}

// ---------------- entry segment: air gap, outer wall, acrylic solid, headspace (:4699-4732) ----------------
// Returns true when the history ended (r.st set), false when the ray entered the water.
template <class S>
__device__ __forceinline__ bool entry_segment(const DevScene& D, Ray& r, S* st) {
    const clr_scene_params& P = D.P;
    float x = r.x, y = r.y, z = r.z, vx = r.vx, vy = r.vy, vz = r.vz;
    const o_cell C = make_cell(P);
    double tdw = o_cyl_hit_finite(x, y, z, vx, vy, vz, P.rout, P.zmin - P.bottom_disc_thickness, P.zwall_top);
    float t = (tdw < 0.5 * (double)CLR_INF_F) ? (float)tdw : CLR_INF_F;
    if (t >= CLR_INF_F * 0.5f) { r.st = 3; return true; }
    x += t * vx; y += t * vy; z += t * vz;
    float nx, ny;
    o_radial_normal(x, y, &nx, &ny);
    float ci = fminf(fmaxf(-o_dot(vx, vy, vz, nx, ny, 0.0f), 0.0f), 1.0f);
    int tir = 0;
    float R = o_fresnel(ci, P.n_air, P.n_acrylic, &tir);
    float a, b, c;
    if (tir || uniform(st) < R || !o_refract(vx, vy, vz, nx, ny, 0.0f, P.n_air, P.n_acrylic, &a, &b, &c)) {
        o_reflect(vx, vy, vz, nx, ny, 0.0f, &a, &b, &c);
        vx = a; vy = b; vz = c; r.cor++; if (tir) r.ctir++;
        x += CLR_EPS_F * nx; y += CLR_EPS_F * ny;
        r.x = x; r.y = y; r.z = z; r.vx = vx; r.vy = vy; r.vz = vz;
        r.st = 1;
        return true;
    }
    vx = a; vy = b; vz = c; x -= CLR_EPS_F * nx; y -= CLR_EPS_F * ny;
    o_bcount bc = {0, 0, 0, 0, 0, 0, 0, 0};
    int sub = 0, nb = 0;
    int where = o_acrylic_solid(st, &C, C.n_air, C.n_bottom_ext, P.zmin, C.Zlow, &x, &y, &z, &vx, &vy, &vz, &r.ap, &bc,
                                &sub, &nb);
    bool ended = false;
    if (where == 2) { r.st = 1; ended = true; }
    else if (where == 3) { r.st = 7; ended = true; }
    else if (where == 5) { r.st = 8; ended = true; }
    else if (where == 4) {
        int hs = 0, hb = 0;
        int hw = o_headspace(st, &C, &x, &y, &z, &vx, &vy, &vz, &r.ap, &bc, &hs, &hb);
        if (hw == 1) r.entered = 1;
        else if (hw == 2) { r.st = 1; ended = true; }
        else if (hw == 3) { r.st = 7; ended = true; }
        else if (hw == 4) { r.st = 6; ended = true; }
        else if (hw == 5) { r.st = 8; ended = true; }
        else { r.pf = OP_HEADSPACE_NO_BOUNDARY; r.pfs = hs; r.st = 4; ended = true; }
    } else if (where != 1) {
        r.pf = (sub == OS_ACRYLIC_BOUNCE_LIMIT) ? OP_ACRYLIC_BOUNCE_LIMIT : OP_ACRYLIC_NO_INTERSECTION;
        r.pfs = sub; r.st = 4; ended = true;
    }
    add_bounces(r, bc);
    r.x = x; r.y = y; r.z = z; r.vx = vx; r.vy = vy; r.vz = vz;
    if (ended) return true;
    r.entered = 1;
    r.phase = PHASE_WATER;
    r.step = 0;
    return false;
}

// ---------------- field lookup for the counter-based stream (sediment model 3) ----------------
// The interpolated field sum_i mu_i g_i(r, z) is linear in the node values, so it equals the bilinear
// interpolation of the node sums G_c = sum_i mu_i g_i[c]. A bin drawn with probability proportional to
// mu_i g_i(r, z) is drawn by composition: a corner c with probability w_c G_c / sum_c' w_c' G_c', then a
// bin from node c's alias table (probability mu_i g_i[c] / G_c). The distribution is the reference's
// (o_sample_local_bin); the work is four node reads and one alias read instead of a pass over all bins.
struct NodeLookup {
    int node[4];
    float wg[2][4];
    float local[2];
};

__device__ __forceinline__ void node_lookup(const DevScene& D, float x, float y, float z, NodeLookup& L) {
    const int NR = D.grid_nr, NZ = D.grid_nz;
    const float R = D.P.rin, zmin = D.P.zmin;
    const float rr = fminf(sqrtf(fmaxf(x * x + y * y, 0.0f)), R);
    float ur = rr * ((float)NR / R) - 0.5f;
    float uz = (z - zmin) * ((float)NZ / (D.grid_zmax - zmin)) - 0.5f;
    ur = fminf(fmaxf(ur, 0.0f), (float)(NR - 1));
    uz = fminf(fmaxf(uz, 0.0f), (float)(NZ - 1));
    int i = (int)ur, k = (int)uz;
    float tr = ur - (float)i, tz = uz - (float)k;
    if (i >= NR - 1) { i = NR - 2; tr = 1.0f; }
    if (k >= NZ - 1) { k = NZ - 2; tz = 1.0f; }
    const int b = i * NZ + k;
    L.node[0] = b; L.node[1] = b + NZ; L.node[2] = b + 1; L.node[3] = b + NZ + 1;
    const float w[4] = {(1.0f - tr) * (1.0f - tz), tr * (1.0f - tz), (1.0f - tr) * tz, tr * tz};
    float lg = 0.0f, lw = 0.0f;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const float2 g = __ldg(&D.node_mu[L.node[c]]);
        L.wg[0][c] = w[c] * g.x;
        L.wg[1][c] = w[c] * g.y;
        lg += L.wg[0][c];
        lw += L.wg[1][c];
    }
    L.local[0] = lg;
    L.local[1] = lw;
}

template <class S>
__device__ __forceinline__ int node_sample_bin(const DevScene& D, S* st, const NodeLookup& L, int ch) {
    if (!(L.local[ch] > 0.0f)) return 0;
    const float target = uniform(st) * L.local[ch];
    int c = -1, last = 0;
    float cum = 0.0f;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const float wq = L.wg[ch][q];
        if (wq > 0.0f) last = q;
        cum += wq;
        if (c < 0 && wq > 0.0f && target < cum) c = q;
    }
    if (c < 0) c = last;
    const int n = D.n_bins;
    const int2* A = D.node_alias + ((size_t)ch * (size_t)(D.grid_nr * D.grid_nz) + (size_t)L.node[c]) * (size_t)n;
    const int j = (int)__umulhi(st->next(), (uint32_t)n);
    const int2 e = __ldg(&A[j]);
    return (uniform(st) < __int_as_float(e.x)) ? j : e.y;
}

// ---------------- one water free-flight step (one iteration of :4734-5066) ----------------
// An iteration is split into its flight part (boundary distances, free path, move, delta-tracking
// acceptance, channel and bin choice, and the cheap outcomes: null collisions, coherent Mie
// scattering, Fresnel reflections at the free surface and the cell wall) and one handler per
// expensive outcome (conditional closure, geometric sphere, spheroid morphology, transmission into
// the headspace or the acrylic wall, bottom disc). The persistent kernel runs both back to back
// (water_step); the wavefront engine runs each handler as its own kernel over a queue of photons.
// Split or not, the arithmetic and the per-ray draw order are those of the reference iteration.
enum : int { WE_NONE = 0, WE_ENDED = 1, WE_COND = 2, WE_GEOM = 3, WE_MORPH = 4, WE_TOP = 5, WE_BOTTOM = 6,
             WE_SIDE = 7 };

__device__ __forceinline__ void apply_moment(const DevScene& D, int pidx, float vinx, float viny, float vinz, float* vx,
                                             float* vy, float* vz) {
    if (D.any_moment && pidx >= 0 && D.moment_mode[pidx])
        moment_constraint(vinx, viny, vinz, vx, vy, vz, (float)D.moment_a[pidx], (float)D.moment_b[pidx]);
}

// ---------------- weighted transport (no reference counterpart) ----------------
// With weight_mode == CLR_WEIGHT_IMPLICIT (counter-based stream only) absorption is never sampled: at an
// absorbing particle the photon always scatters and its weight is multiplied by the survival
// probability (the particle albedo in the conditional closure, exp(-alpha chord) per internal chord of a
// sphere or spheroid, exp(-mu_a travel) per water flight). The detector tallies then sum weights, and the
// expected tallies equal the analog ones. A photon whose weight falls below roulette_threshold survives
// with probability w / roulette_survival and then carries roulette_survival, else it ends with status
// CLR_STATUS_ROULETTE: an unbiased cut of the long, low-weight tail.
__device__ __forceinline__ bool weighted_run(const DevScene& D) { return D.weight_mode == CLR_WEIGHT_IMPLICIT; }

// Russian roulette after a weight change; true when the photon was killed.
template <class S>
__device__ __forceinline__ bool roulette(const DevScene& D, Ray& r, S* st) {
    if (!(r.w < D.roulette_threshold)) return false;
    if (uniform(st) * D.roulette_survival < r.w) {
        r.w = D.roulette_survival;
        return false;
    }
    r.w = 0.0f;
    r.st = CLR_STATUS_ROULETTE;
    return true;
}

// True when the straight segment of length t from (x, y, z) along v stays inside the water: the
// cylinder and the half-space above the bottom are convex, so their test is the endpoint's; the free
// surface height grows with the radius in every surface model, so the segment stays below it when its
// highest point lies below the surface height at its smallest radius. Margins (tens of nm) absorb FP32
// rounding; a segment that fails the test takes the exact boundary computation.
__device__ __forceinline__ bool flight_clear(const clr_scene_params& P, float x, float y, float z, float vx, float vy,
                                             float vz, float t) {
    if (!(t < 1.0f)) return false;
    const float x1 = x + t * vx, y1 = y + t * vy, z1 = z + t * vz;
    const float R = P.rin;
    if (!(x1 * x1 + y1 * y1 < R * R * 0.99999f)) return false;
    if (!(z1 > P.zmin + 1e-6f)) return false;
    float rmin2 = fminf(x * x + y * y, x1 * x1 + y1 * y1);
    const float a = vx * vx + vy * vy;
    if (a > 1e-20f) {
        const float ts = -(x * vx + y * vy) / a;
        if (ts > 0.0f && ts < t) {
            const float xs = x + ts * vx, ys = y + ts * vy;
            rmin2 = fminf(rmin2, xs * xs + ys * ys);
        }
    }
    const float zs = o_surface_z(sqrtf(rmin2), 0.0f, P.zmean, R, P.free_surface_model, P.vortex_delta_h,
                                 P.vortex_core_radius);
    return fmaxf(z, z1) < zs - 1e-6f;
}

// ---------------- light-history diagnostics (observational: no random draw, no state change) ----------------
// Heat maps: every 10 um along a water segment one count in the x-y and z-y maps (:3296-3310).
__device__ void light_heat_segment(const LightDiag& L, float x0, float y0, float z0, float vx, float vy, float vz,
                                   float dist, float Rin, float zmin) {
    const int vis = L.vis;
    if (vis <= 0 || dist <= 0.0f) return;
    const float spacing = 1.0e-5f;
    int n = (int)ceilf(dist / spacing);
    if (n < 1) n = 1;
    if (n > 20000) n = 20000;
    for (int k = 1; k <= n; ++k) {
        float f = (float)k / (float)n;
        float x = x0 + vx * dist * f, y = y0 + vy * dist * f, z = z0 + vz * dist * f;
        int ix = (int)(((x + Rin) / (2.0f * Rin)) * vis);
        int iy = vis - 1 - (int)(((y + Rin) / (2.0f * Rin)) * vis);
        int iz = (int)(((z - zmin) / (L.zvis - zmin)) * vis);
        if (ix >= 0 && ix < vis && iy >= 0 && iy < vis) atomicAdd(&L.heat_xy[iy * vis + ix], 1.0f);
        if (iz >= 0 && iz < vis && iy >= 0 && iy < vis) atomicAdd(&L.heat_zy[iy * vis + iz], 1.0f);
    }
}

__device__ __forceinline__ int light_clip_axis(double p, double d, double lo, double hi, double* t0, double* t1) {
    if (fabs(d) < 1.0e-30f) return (p >= lo && p <= hi) ? 1 : 0;
    double a = (lo - p) / d, b = (hi - p) / d;
    if (a > b) { double q = a; a = b; b = q; }
    *t0 = fmax(*t0, a); *t1 = fmin(*t1, b);
    return *t1 >= *t0;
}

// Exact track-length deposition of one water segment by a 3-D voxel traversal in FP64, with the
// reference's endpoint-snap tolerance and integrity counters (:3318-3400); representative rays keep their
// clipped segments.
__device__ void light_segment(const LightDiag& L, uint32_t gid, float Rin, float zmin, float x0, float y0,
                              float z0, float vx, float vy, float vz, float dist, int particle_order) {
    if (!(dist > 0.0f) || !isfinite(dist)) return;
    const int nx = L.nx, ny = L.ny, nz = L.nz;
    const float zmax = L.zmax;
    if (nx <= 0 || ny <= 0 || nz <= 0 || !(zmax > zmin)) { atomicAdd(L.err_count, 1u); return; }
    const double xmin = -(double)Rin, ymin = -(double)Rin;
    double c0 = 0.0, c1 = 1.0;
    if (!light_clip_axis(x0, (double)vx * (double)dist, -Rin, Rin, &c0, &c1) ||
        !light_clip_axis(y0, (double)vy * (double)dist, -Rin, Rin, &c0, &c1) ||
        !light_clip_axis(z0, (double)vz * (double)dist, zmin, zmax, &c0, &c1))
        return;
    const double ax = x0 + (double)vx * (double)dist * c0, ay = y0 + (double)vy * (double)dist * c0,
                 az = z0 + (double)vz * (double)dist * c0;
    const double x1 = x0 + (double)vx * (double)dist * c1, y1 = y0 + (double)vy * (double)dist * c1,
                 z1 = z0 + (double)vz * (double)dist * c1;
    const double clipped = dist * (c1 - c0);
    if (!(clipped > 0.0f)) return;
    atomicAdd(L.seg_total, clipped);
    atomicAdd(L.seg_count, 1ull);
    if ((int)gid < L.rep_rays && L.max_segments > 0) {
        const int slot = L.tcount[gid];
        if (slot < L.max_segments) {
            const int q = (int)gid * L.max_segments + slot;
            L.tx0[q] = (float)ax; L.ty0[q] = (float)ay; L.tz0[q] = (float)az;
            L.tx1[q] = (float)x1; L.ty1[q] = (float)y1; L.tz1[q] = (float)z1;
            L.torder[q] = particle_order;
            L.tcount[gid] = slot + 1;
        } else {
            L.toverflow[gid] = 1;
        }
    }
    const double dx = (2.0 * (double)Rin) / nx, dy = (2.0 * (double)Rin) / ny, dz = ((double)zmax - (double)zmin) / nz;
    int ix = (int)floor((ax - xmin) / dx), iy = (int)floor((ay - ymin) / dy), iz = (int)floor((az - zmin) / dz);
    if (ix < 0) ix = 0;
    if (ix >= nx) ix = nx - 1;
    if (iy < 0) iy = 0;
    if (iy >= ny) iy = ny - 1;
    if (iz < 0) iz = 0;
    if (iz >= nz) iz = nz - 1;
    const double sx = x1 - ax, sy = y1 - ay, sz = z1 - az;
    const int stepx = (sx > 0.0f) ? 1 : ((sx < 0.0f) ? -1 : 0);
    const int stepy = (sy > 0.0f) ? 1 : ((sy < 0.0f) ? -1 : 0);
    const int stepz = (sz > 0.0f) ? 1 : ((sz < 0.0f) ? -1 : 0);
    double bx = xmin + (double)(stepx > 0 ? ix + 1 : ix) * dx;
    double by = ymin + (double)(stepy > 0 ? iy + 1 : iy) * dy;
    double bz = zmin + (double)(stepz > 0 ? iz + 1 : iz) * dz;
    double tmx = (stepx == 0) ? CLR_INF_F : (bx - ax) / sx;
    double tmy = (stepy == 0) ? CLR_INF_F : (by - ay) / sy;
    double tmz = (stepz == 0) ? CLR_INF_F : (bz - az) / sz;
    if (tmx < 0.0f) tmx = 0.0f;
    if (tmy < 0.0f) tmy = 0.0f;
    if (tmz < 0.0f) tmz = 0.0f;
    double u = 0.0, deposited = 0.0;
    const float tol = 2.0e-6f;
    const int max_steps = nx + ny + nz + 8;
    for (int k = 0; k < max_steps && u < 1.0f; ++k) {
        if (ix < 0 || ix >= nx || iy < 0 || iy >= ny || iz < 0 || iz >= nz) {
            if (u >= 1.0f - tol) { atomicAdd(L.adj_count, 1u); u = 1.0f; break; }
            atomicAdd(L.err_count, 1u);
            break;
        }
        double un = fmin(1.0, fmin(tmx, fmin(tmy, tmz)));
        if (un < 1.0f && un >= 1.0f - tol) { un = 1.0f; atomicAdd(L.adj_count, 1u); }
        if (un < u) {
            if (u - un <= tol) { un = u; atomicAdd(L.adj_count, 1u); }
            else { atomicAdd(L.err_count, 1u); break; }
        }
        const double length = (un - u) * clipped;
        if (length > 0.0f) {
            const int q = (iz * ny + iy) * nx + ix;
            atomicAdd(&L.total[q], (float)length);
            if (particle_order > 0) atomicAdd(&L.post[q], (float)length);
            deposited += length;
        }
        if (un >= 1.0f) { u = 1.0f; break; }
        const double eps = 8.0 * 2.2204460492503131e-16 * fmax(1.0, fabs(un));
        if (tmx <= un + eps) { ix += stepx; tmx = (xmin + (double)(stepx > 0 ? ix + 1 : ix) * dx - ax) / sx; }
        if (tmy <= un + eps) { iy += stepy; tmy = (ymin + (double)(stepy > 0 ? iy + 1 : iy) * dy - ay) / sy; }
        if (tmz <= un + eps) { iz += stepz; tmz = ((double)zmin + (double)(stepz > 0 ? iz + 1 : iz) * dz - az) / sz; }
        u = un;
    }
    if (u < 1.0f - tol) atomicAdd(L.err_count, 1u);
    atomicAdd(L.dep_total, deposited);
}

// A scatter-event site into its voxel (:3409-3438).
__device__ void light_event(const LightDiag& L, uint32_t gid, float Rin, float zmin, float x, float y, float z) {
    atomicAdd(L.event_total, 1ull);
    const float zmax = L.zmax;
    const float tol = 2.0e-6f * fmaxf(2.0f * Rin, zmax - zmin);
    if (!isfinite(x) || !isfinite(y) || !isfinite(z) || x < -Rin - tol || x > Rin + tol || y < -Rin - tol ||
        y > Rin + tol || z < zmin - tol || z > zmax + tol) {
        const unsigned prev = atomicAdd(L.outside, 1u);
        if (prev == 0u) {
            L.outside[1] = __float_as_uint(x); L.outside[2] = __float_as_uint(y); L.outside[3] = __float_as_uint(z);
            L.outside[4] = gid; L.outside[5] = __float_as_uint(tol); L.outside[6] = 1u;
        }
        atomicAdd(L.err_count, 1u);
        return;
    }
    const int nx = L.nx, ny = L.ny, nz = L.nz;
    int ix = (int)floorf(((x + Rin) / (2.0f * Rin)) * nx);
    int iy = (int)floorf(((y + Rin) / (2.0f * Rin)) * ny);
    int iz = (int)floorf(((z - zmin) / (zmax - zmin)) * nz);
    int adjusted = 0;
    if (ix < 0) { ix = 0; adjusted = 1; } else if (ix >= nx) { ix = nx - 1; adjusted = 1; }
    if (iy < 0) { iy = 0; adjusted = 1; } else if (iy >= ny) { iy = ny - 1; adjusted = 1; }
    if (iz < 0) { iz = 0; adjusted = 1; } else if (iz >= nz) { iz = nz - 1; adjusted = 1; }
    if (adjusted) atomicAdd(L.adj_count, 1u);
    const int q = (iz * ny + iy) * nx + ix;
    atomicAdd(&L.event_weight[q], 1.0f);
    atomicAdd(&L.event_count[q], 1u);
}

// Flight part. Returns WE_NONE when the iteration completed (the photon stays in the water),
// WE_ENDED when the history ended, else the handler that completes the iteration (*ev_pidx is the
// bin of a particle event). Position and direction are stored in r in every case.
template <class S, bool kLight = true>
__device__ __forceinline__ int water_flight(const DevScene& D, Ray& r, S* st, S* opt, unsigned long long* cstats,
                                            int* ev_pidx, uint32_t gid) {
    const clr_scene_params& P = D.P;
    if (r.step >= (int)P.max_iterations) { r.pf = OP_ITERATION_LIMIT; r.pfs = OS_ITERATION_LIMIT; r.st = 4; return WE_ENDED; }
    r.step++;
    r.steps++;
    const int TM = P.sediment_model, FSM = P.free_surface_model;
    const float RIN = P.rin, ZMIN = P.zmin, ZMEAN = P.zmean, ZTOP = P.zwall_top, DH = P.vortex_delta_h,
                CORE = P.vortex_core_radius;
    float x = r.x, y = r.y, z = r.z, vx = r.vx, vy = r.vy, vz = r.vz;
    int res = WE_NONE;
    do {
        if (!isfinite(x) || !isfinite(y) || !isfinite(z)) { r.pf = OP_NONFINITE_POSITION; r.pfs = OS_NONFINITE_POSITION; r.st = 4; res = WE_ENDED; break; }
        if (!isfinite(vx) || !isfinite(vy) || !isfinite(vz)) { r.pf = OP_NONFINITE_DIRECTION; r.pfs = OS_NONFINITE_DIRECTION; r.st = 4; res = WE_ENDED; break; }
        float zsurf_here = o_surface_z(x, y, ZMEAN, RIN, FSM, DH, CORE);
        if (z <= ZMIN || z >= zsurf_here) { r.st = 2; res = WE_ENDED; break; }
        bool outside;
        if constexpr (kCounterStream<S>) {
            outside = x * x + y * y > RIN * RIN * (1.0f + 8.0f * 1.1920928955078125e-7f);
        } else {
            double rr2w = (double)x * (double)x + (double)y * (double)y, ri2w = (double)RIN * (double)RIN;
            double water_tol = 8.0 * 1.1920928955078125e-7 * ri2w;
            outside = rr2w > ri2w + water_tol;
        }
        if (outside) { r.pf = OP_INVALID_MEDIUM; r.pfs = OS_WATER_OUTSIDE; r.st = 4; res = WE_ENDED; break; }
        const float MU_GEOM = D.mu_geom_f, MU_WAVE = D.mu_wave_f;
        float MU_TOTAL = MU_GEOM + MU_WAVE;
        // counter-based streams with node tables use the node-sum majorant (never above the reference's)
        const bool node_fast = kCounterStream<S> && TM == 3 && D.node_alias != nullptr;
        float MU_TRACK = (TM == 0) ? MU_TOTAL : node_fast ? D.node_major : (D.sed_major_f[0] + D.sed_major_f[1]);
        int axial_top = 0, axial_bottom = 0, do_particle = 0;
        float travel = 0.0f;
        bool lazy = false;
        float fp_pre = CLR_INF_F;
        if constexpr (kCounterStream<S>) {
            // Counter-based streams draw the free path first; when the whole segment provably stays in
            // the water the boundary distances (FP64 wall and free-surface roots) are not needed.
            if (MU_TRACK > 0.0f) {
                const float u = fmaxf(uniform(st), 1e-12f);
                fp_pre = -logf(u) / MU_TRACK;
                if (flight_clear(P, x, y, z, vx, vy, vz, fp_pre)) { do_particle = 1; travel = fp_pre; lazy = true; }
            }
        }
        if (!lazy) {
            float tside, ttop, tbottom = CLR_INF_F;
            if constexpr (kCounterStream<S>) {
                tside = f_bore_wall_hit(x, y, z, vx, vy, vz, RIN, ZMIN, ZTOP);
                if (tside < 0.0f) { r.pf = OP_INVALID_MEDIUM; r.pfs = OS_WATER_OUTSIDE; r.st = 4; res = WE_ENDED; break; }
                ttop = f_surface_hit(x, y, z, vx, vy, vz, ZMEAN, RIN, FSM, DH, CORE);
            } else {
                double tsided = o_bore_wall_hit(x, y, z, vx, vy, vz, RIN, ZMIN, ZTOP);
                if (tsided < 0.0) { r.pf = OP_INVALID_MEDIUM; r.pfs = OS_WATER_OUTSIDE; r.st = 4; res = WE_ENDED; break; }
                tside = (tsided < 0.5 * (double)CLR_INF_F) ? (float)tsided : CLR_INF_F;
                ttop = o_surface_hit(x, y, z, vx, vy, vz, ZMEAN, RIN, FSM, DH, CORE);
            }
            if (vz < -1e-14f) tbottom = (ZMIN - z) / vz;
            if (!(ttop > 0.0f)) ttop = CLR_INF_F;
            if (!(tbottom > 0.0f)) tbottom = CLR_INF_F;
            axial_top = (ttop <= tbottom && ttop < tside);
            axial_bottom = (tbottom < ttop && tbottom < tside);
            float tbound = axial_top ? ttop : (axial_bottom ? tbottom : tside);
            if (tbound >= CLR_INF_F * 0.5f) { r.pf = OP_WATER_NO_BOUNDARY; r.pfs = OS_WATER_NO_BOUNDARY; r.st = 4; res = WE_ENDED; break; }
            float freep = CLR_INF_F;
            if (tbound > 0.0f && MU_TRACK > 0.0f) {
                if constexpr (kCounterStream<S>) {
                    freep = fp_pre;
                } else {
                    float u = fmaxf(uniform(st), 1e-12f);
                    freep = -logf(u) / MU_TRACK;
                }
            }
            do_particle = freep < tbound;
            travel = do_particle ? freep : tbound;
        }
        // absorption by the water itself (no reference counterpart; skipped, with no draw, when mu_a is 0)
        bool water_absorbed = false;
        if (P.water_absorption > 0.0f) {
            if (weighted_run(D)) {
                r.w *= expf(-P.water_absorption * travel);
                if (roulette(D, r, st)) { res = WE_ENDED; break; }
            } else {
                const float da = -logf(fmaxf(uniform(st), 1e-12f)) / P.water_absorption;
                if (da < travel) { travel = da; water_absorbed = true; }
            }
        }
        if (kLight && D.light) {  // the segment about to be flown (:4763-4772): heat maps for every ray, voxels for the first
            const LightDiag& LD = *D.light;
            if (LD.vis > 0) light_heat_segment(LD, x, y, z, vx, vy, vz, travel, RIN, ZMIN);
            if (LD.voxels && gid < (uint32_t)LD.max_rays) light_segment(LD, gid, RIN, ZMIN, x, y, z, vx, vy, vz, travel, r.ic);
        }
        x += travel * vx; y += travel * vy; z += travel * vz;
        r.wp += travel;
        if (water_absorbed) { r.st = 5; res = WE_ENDED; break; }
        if (do_particle && !lazy) {
            bool end_out;
            if constexpr (kCounterStream<S>) {
                end_out = x * x + y * y > RIN * RIN * (1.0f + 8.0f * 1.1920928955078125e-7f);
            } else {
                double endpoint_r2 = (double)x * x + (double)y * y, ri2w = (double)RIN * (double)RIN;
                end_out = endpoint_r2 > ri2w + 8.0 * 1.1920928955078125e-7 * ri2w;
            }
            if (end_out || z < ZMIN - CLR_EPS_F || z > o_surface_z(x, y, ZMEAN, RIN, FSM, DH, CORE) + CLR_EPS_F) {
                r.pf = OP_INVALID_MEDIUM; r.pfs = OS_WATER_OUTSIDE; r.st = 4; res = WE_ENDED; break;
            }
        }
        if (do_particle) {
            const o_field F = make_field(D);
            float LOCAL_GEOM = MU_GEOM, LOCAL_WAVE = MU_WAVE, LOCAL_TOTAL = MU_TOTAL;
            NodeLookup NL;
            if (TM != 0) {
                if (node_fast) {
                    node_lookup(D, x, y, z, NL);
                    LOCAL_GEOM = NL.local[0]; LOCAL_WAVE = NL.local[1];
                } else if (TM == 3) {
                    const o_grid_w gw = o_grid_weights(&F, x, y, z);
                    double lg = 0.0, lw = 0.0;
                    for (int i = 0; i < D.n_bins; ++i) {
                        double sc = o_grid_sample_w(&F, gw, i);
                        lg += D.trace_geom[i] * sc;
                        lw += D.trace_wave[i] * sc;
                    }
                    LOCAL_GEOM = (float)lg; LOCAL_WAVE = (float)lw;
                } else {
                    double lg = 0.0, lw = 0.0;
                    for (int i = 0; i < D.n_bins; ++i) {
                        double sc = o_local_scale(&F, i, x, y, z);
                        lg += D.trace_geom[i] * sc;
                        lw += D.trace_wave[i] * sc;
                    }
                    LOCAL_GEOM = (float)lg; LOCAL_WAVE = (float)lw;
                }
                LOCAL_TOTAL = LOCAL_GEOM + LOCAL_WAVE;
                if (!(LOCAL_TOTAL > 0.0f)) { r.nulls++; break; }
                float slack = 64.0f * 1.1920928955078125e-7f * fmaxf(fabsf(MU_TRACK), 1.0f);
                if (LOCAL_TOTAL > MU_TRACK + slack) { r.pf = OP_MAJORANT_VIOLATION; r.pfs = OS_MAJORANT; r.st = 4; res = WE_ENDED; break; }
                float pacc = LOCAL_TOTAL / fmaxf(MU_TRACK, 1e-30f);
                if (pacc > 1.0f) pacc = 1.0f;
                if (uniform(st) >= pacc) { r.nulls++; break; }
            }
            r.ic++;
            if (kLight && D.light && D.light->voxels && gid < (uint32_t)D.light->max_rays)
                light_event(*D.light, gid, RIN, ZMIN, x, y, z);
            const float vinx = vx, viny = vy, vinz = vz;
            const int COND = (P.event_model == 4 || P.event_model == 5);
            const float COHERENT = fminf(fmaxf(D.coherent_f, 0.0f), 1.0f);
            int use_wave = (LOCAL_WAVE > 0.0f && uniform(st) * LOCAL_TOTAL >= LOCAL_GEOM);
            int sel = -1;
            if (COND) {
                if (TM == 0) sel = o_sample_cdf(st, use_wave ? D.wcdf : D.gcdf, D.n_bins);
                else if (node_fast) sel = node_sample_bin(D, st, NL, use_wave);
                else sel = o_sample_local_bin(st, &F, use_wave ? D.trace_wave : D.trace_geom, x, y, z,
                                              (double)(use_wave ? LOCAL_WAVE : LOCAL_GEOM));
            }
            if (COND && D.k[sel] > 0.0) {
                if (D.pk[sel] == 0.0f) { r.pf = OP_OTHER; r.pfs = 9003; r.st = 4; atomicAdd(&cstats[8], 1ull); res = WE_ENDED; break; }
                *ev_pidx = sel;
                res = WE_COND;
                break;
            }
            if (use_wave) {
                if (COND) atomicAdd(&cstats[0], 1ull);
                r.wic++;
                int pidx = sel >= 0 ? sel
                                    : (TM == 0) ? o_sample_cdf(st, D.wcdf, D.n_bins)
                                    : node_fast ? node_sample_bin(D, st, NL, 1)
                                                : o_sample_local_bin(st, &F, D.trace_wave, x, y, z, (double)LOCAL_WAVE);
                int coherent = (COHERENT >= 1.0f) || (uniform(opt) < COHERENT);
                if (coherent) {
                    r.wcoh++;
                    o_mie_direction(opt, D.phase_cdf, D.theta, D.nt, pidx, &vx, &vy, &vz, D.phase_guide);
                    if (COND) { atomicAdd(&cstats[4], 1ull); atomicAdd(&cstats[7], 1ull); }
                    apply_moment(D, pidx, vinx, viny, vinz, &vx, &vy, &vz);
                    if constexpr (kLight) *ev_pidx = pidx;  // the diagnostic callers' provenance of the event
                    break;
                }
                r.wmorph++;
                *ev_pidx = pidx;
                res = WE_MORPH;
                break;
            }
            if (COND) atomicAdd(&cstats[0], 1ull);
            r.gic++;
            *ev_pidx = sel >= 0 ? sel
                                : (TM == 0) ? o_sample_cdf(st, D.gcdf, D.n_bins)
                                : node_fast ? node_sample_bin(D, st, NL, 0)
                                            : o_sample_local_bin(st, &F, D.trace_geom, x, y, z, (double)LOCAL_GEOM);
            res = WE_GEOM;
            break;
        }
        if (axial_bottom) { res = WE_BOTTOM; break; }
        if (axial_top) {
            float a, b, c;
            int tir = 0;
            float snx = 0.0f, sny = 0.0f, snz = -1.0f;
            o_surface_normal(x, y, RIN, FSM, DH, CORE, &snx, &sny, &snz);
            float ci = fminf(fmaxf(-o_dot(vx, vy, vz, snx, sny, snz), 0.0f), 1.0f);
            float R = o_fresnel(ci, P.n_water, P.n_air, &tir);
            if (tir || uniform(st) < R || !o_refract(vx, vy, vz, snx, sny, snz, P.n_water, P.n_air, &a, &b, &c)) {
                o_reflect(vx, vy, vz, snx, sny, snz, &a, &b, &c);
                vx = a; vy = b; vz = c; r.tr++; if (tir) r.ttir++;
                if (!o_surface_offset(&x, &y, &z, snx, sny, snz, RIN, ZMIN, ZMEAN, FSM, DH, CORE)) {
                    r.pf = OP_INVALID_MEDIUM; r.pfs = OS_WATER_OUTSIDE; r.st = 4; res = WE_ENDED;
                }
                break;
            }
            vx = a; vy = b; vz = c;
            x -= CLR_EPS_F * snx; y -= CLR_EPS_F * sny; z -= CLR_EPS_F * snz;
            res = WE_TOP;
            break;
        }
        // water -> acrylic at the cylinder wall (:5038-5065)
        {
            float nx, ny;
            o_radial_normal(x, y, &nx, &ny);
            float ci = fminf(fmaxf(o_dot(vx, vy, vz, nx, ny, 0.0f), 0.0f), 1.0f);
            int tir = 0;
            float R = o_fresnel(ci, P.n_water, P.n_acrylic, &tir);
            float a, b, c;
            if (tir || uniform(st) < R || !o_refract(vx, vy, vz, -nx, -ny, 0.0f, P.n_water, P.n_acrylic, &a, &b, &c)) {
                o_reflect(vx, vy, vz, nx, ny, 0.0f, &a, &b, &c);
                vx = a; vy = b; vz = c; r.cir++; if (tir) r.ctir++;
                x -= CLR_EPS_F * nx; y -= CLR_EPS_F * ny;
                break;
            }
            vx = a; vy = b; vz = c; x += CLR_EPS_F * nx; y += CLR_EPS_F * ny;
            res = WE_SIDE;
        }
    } while (false);
    r.x = x; r.y = y; r.z = z; r.vx = vx; r.vy = vy; r.vz = vz;
    return res;
}

// ---- handlers: each completes the iteration its flight part started; true when the history ended ----

// Conditional closures complete either a flight whose bin is absorbing (CK_FLIGHT, :4818-4830) or a
// geometric event whose sampled sphere does not fit in the water (CK_GEOM, :4890-4905).
enum : int { CK_FLIGHT = 0, CK_GEOM = 1 };

// Completes the iteration of a finished closure with its result h: 0 when the photon continues in the
// water, 1 when the history ended.
template <class S>
__device__ __forceinline__ int closure_finish(const DevScene& D, Ray& r, S* opt, int pidx, int kind, const Hist& h) {
    float x = r.x, y = r.y, z = r.z, vx = r.vx, vy = r.vy, vz = r.vz;
    const float vinx = vx, viny = vy, vinz = vz;
    bool ended = false;
    do {
        if (kind == CK_FLIGHT) {
            if (h.status != 1 && h.status != 2) { r.pf = h.failure ? h.failure : OP_OTHER; r.pfs = h.subcode; r.st = 4; ended = true; break; }
        } else {
            if (h.status != 1) { r.pf = h.failure ? h.failure : OP_OTHER; r.pfs = h.subcode; r.st = 4; ended = true; break; }
        }
        x = h.x; y = h.y; z = h.z; vx = h.vx; vy = h.vy; vz = h.vz;
        r.pc.reflections += h.pc.reflections; r.pc.entry_reflections += h.pc.entry_reflections;
        r.pc.internal_reflections += h.pc.internal_reflections; r.pc.absorptions += h.pc.absorptions;
        if (kind == CK_GEOM) r.gic--;
        if (h.channel == 0) r.gic++;
        else { r.wic++; if (h.channel == 1) r.wcoh++; else r.wmorph++; }
        if (kind == CK_FLIGHT && h.status == 2) { r.st = 5; ended = true; break; }
        apply_moment(D, pidx, vinx, viny, vinz, &vx, &vy, &vz);
        if (kind == CK_FLIGHT && weighted_run(D) && roulette(D, r, opt)) ended = true;
    } while (false);
    r.x = x; r.y = y; r.z = z; r.vx = vx; r.vy = vy; r.vz = vz;
    return ended ? 1 : 0;
}

// Runs (part of) a closure. Returns 0 when the iteration ended with the photon in the water, 1 when the
// history ended, 2 when the closure continues (state in *cs; with budget 0 it always finishes).
template <class S>
__device__ __forceinline__ int closure_visit(const DevScene& D, Ray& r, S* opt, unsigned long long* cstats, int pidx,
                                             int kind, CondState* cs, int budget) {
    const clr_scene_params& P = D.P;
    const float COHERENT = fminf(fmaxf(D.coherent_f, 0.0f), 1.0f);
    Hist h;
    const int done = conditional_interaction(
        opt, &h, pidx, D.qsca[pidx], D.qext[pidx], P.n_water, D.pn[pidx], D.pk[pidx], P.wavelength, P.rough_alpha,
        D.prad[pidx], P.spheroid_aspect, P.orientation_model, P.orientation_kappa, P.max_particle_bounces, COHERENT,
        D.phase_cdf, D.theta, D.phase_guide, D.nt, r.x, r.y, r.z, r.vx, r.vy, r.vz, P.rin, P.zmin, P.zmean,
        P.free_surface_model,
        P.vortex_delta_h, P.vortex_core_radius, kind == CK_GEOM ? P.conditional_retries - 1 : P.conditional_retries,
        cstats, cs, budget, (kind == CK_FLIGHT && weighted_run(D)) ? &r.w : nullptr, closure_trial_tag(r.ic));
    if (!done) return 2;
    return closure_finish(D, r, opt, pidx, kind, h);
}

// Warp-cooperative closure (counter-based stream only; called by all 32 lanes of a warp with the same
// photon). The setup draws from the photon's own stream, identically in every lane; then the warp runs 32
// trials at a time, trial t on its own substream of the photon's Philox key (counter word 2 tagged with
// the event number and t). The trials are independent and identically distributed, so the lowest-index
// trial that ends the closure has the distribution of the serial loop's result, and the counters count
// exactly the trials the serial loop would have run. Same returns as closure_visit; only lane 0 adds the
// trial counters.
__device__ __forceinline__ Hist shfl_hist(const Hist& h, int src) {
    static_assert(sizeof(Hist) % 4 == 0, "Hist is moved as 32-bit words");
    constexpr int kWords = (int)(sizeof(Hist) / 4);
    uint32_t wv[kWords];
    memcpy(wv, &h, sizeof(Hist));
#pragma unroll
    for (int k = 0; k < kWords; ++k) wv[k] = __shfl_sync(0xffffffffu, wv[k], src);
    Hist o;
    memcpy(&o, wv, sizeof(Hist));
    return o;
}
__device__ __forceinline__ int closure_visit_warp(const DevScene& D, Ray& r, PhiloxStream* opt,
                                                  unsigned long long* cstats, int pidx, int kind, CondState* cs,
                                                  int budget) {
    const clr_scene_params& P = D.P;
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    unsigned long long stats[CLR_N_CONDITIONAL_STATS] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    const int max_trials = kind == CK_GEOM ? P.conditional_retries - 1 : P.conditional_retries;
    Hist h;
    int done = 0;
    if (!cs->started)
        done = closure_setup(opt, &h, D.qsca[pidx], D.qext[pidx], D.pk[pidx], max_trials, stats, cs,
                             (kind == CK_FLIGHT && weighted_run(D)) ? &r.w : nullptr);
    if (!done) {
        const double qs = D.qsca[pidx];
        ClosureIn c;
        c.cdf = D.phase_cdf; c.theta = D.theta; c.guide = D.phase_guide;
        c.wave = qs > 0.0 ? fmax(qs - 1.0, 0.0) / qs : 0.0;
        c.nm = P.n_water; c.nr = D.pn[pidx]; c.ki = D.pk[pidx]; c.wl = P.wavelength; c.rough = P.rough_alpha;
        c.radius = D.prad[pidx]; c.aspect = P.spheroid_aspect; c.kappa = P.orientation_kappa;
        c.coherent = fminf(fmaxf(D.coherent_f, 0.0f), 1.0f);
        c.x = r.x; c.y = r.y; c.z = r.z; c.vx = r.vx; c.vy = r.vy; c.vz = r.vz;
        c.rin = P.rin; c.zmin = P.zmin; c.zmean = P.zmean; c.delta = P.vortex_delta_h; c.core = P.vortex_core_radius;
        c.pidx = pidx; c.orientation = P.orientation_model; c.max_bounces = P.max_particle_bounces; c.nt = D.nt;
        c.surface = P.free_surface_model;
        const int end = (budget > 0 && max_trials - cs->trial > budget) ? cs->trial + budget : max_trials;
        const uint32_t tag = closure_trial_tag(r.ic);
        for (int base = cs->trial; base < end && !done; base += 32) {
            const int t = base + lane;
            int res = 0;
            if (t < end) {
                PhiloxStream ts = *opt;
                ts.c2 = tag | (uint32_t)t;
                ts.draw = 0u;
                ts.idx = 4;
                res = closure_trial(&ts, c, cs->target, &h);
            }
            const unsigned term = __ballot_sync(FULL, res == 1);
            const unsigned miss = __ballot_sync(FULL, res == -1), nofit = __ballot_sync(FULL, res == -2);
            const int win = term ? __ffs(term) - 1 : 32;
            const unsigned before = win < 32 ? ((1u << win) - 1u) : FULL;
            stats[0] += (unsigned long long)(term ? win + 1 : min(32, end - base));
            stats[1] += (unsigned long long)__popc(miss & before);
            stats[2] += (unsigned long long)__popc(nofit & before);
            if (term) {
                h = shfl_hist(h, win);
                if (h.status != 1 && h.status != 2) {
                    ++stats[8];
                } else {
                    ++stats[3 + h.channel];
                    ++stats[h.status == 2 ? 6 : 7];
                }
                done = 1;
            }
        }
        if (!done) {
            if (end < max_trials) cs->trial = end;
            else { h = closure_exhausted(stats); done = 1; }
        }
    }
    if (lane == 0) {
#pragma unroll
        for (int i = 0; i < CLR_N_CONDITIONAL_STATS; ++i)
            if (stats[i]) atomicAdd(cstats + i, stats[i]);
    }
    if (!done) return 2;
    return closure_finish(D, r, opt, pidx, kind, h);
}

template <class S>
__device__ __forceinline__ bool water_cond(const DevScene& D, Ray& r, S* opt, unsigned long long* cstats, int sel) {
    CondState cs = cond_start();
    return closure_visit(D, r, opt, cstats, sel, CK_FLIGHT, &cs, 0) == 1;
}

// Geometric event up to the closure: returns 0 (iteration done, photon in water), 1 (history ended) or
// 3 (the sampled sphere does not fit and the closure completes the event).
template <class S>
__device__ __forceinline__ int water_geom_visit(const DevScene& D, Ray& r, S* opt, unsigned long long* cstats,
                                                int pidx) {
    const clr_scene_params& P = D.P;
    const float RIN = P.rin, ZMIN = P.zmin, ZMEAN = P.zmean, DH = P.vortex_delta_h, CORE = P.vortex_core_radius;
    const int FSM = P.free_surface_model;
    float x = r.x, y = r.y, z = r.z, vx = r.vx, vy = r.vy, vz = r.vz;
    const float vinx = vx, viny = vy, vinz = vz;
    const int COND = (P.event_model == 4 || P.event_model == 5);
    int res = 0;
    do {
        float prad = D.prad[pidx];
        float srho, sphi, sgx, sgy, sgz;
        o_sphere_geometry(opt, prad, x, y, z, vx, vy, vz, &srho, &sphi, &sgx, &sgy, &sgz);
        double dscx = 0.0, dscy = 0.0, dscz = 0.0;
        float fcx = 0.0f, fcy = 0.0f, fcz = 0.0f;
        int accessible;
        if constexpr (kCounterStream<S>) {
            fcx = x - prad * sgx; fcy = y - prad * sgy; fcz = z - prad * sgz;
            accessible = f_sphere_accessible(fcx, fcy, fcz, prad, RIN, ZMIN, ZMEAN, FSM, DH, CORE);
        } else {
            dscx = (double)x - (double)prad * (double)sgx;
            dscy = (double)y - (double)prad * (double)sgy;
            dscz = (double)z - (double)prad * (double)sgz;
            accessible = o_sphere_accessible(dscx, dscy, dscz, (double)prad, RIN, ZMIN, ZMEAN, FSM, DH, CORE);
        }
        if (!accessible && COND) {
            atomicAdd(&cstats[2], 1ull);
            res = 3;
            break;
        }
        if (!accessible) { r.ic--; r.gic--; r.nulls++; break; }
        float ipath = 0.0f;
        int ppc = 0, pps = 0, pmb = 0, pmo = 0;
        int ps;
        if constexpr (kCounterStream<S>)
            ps = f_sphere_sampled(opt, P.n_water, D.pn[pidx], D.pk[pidx], P.wavelength, P.rough_alpha, prad,
                                  P.max_particle_bounces, sgx, sgy, sgz, fcx, fcy, fcz, &x, &y, &z, &vx, &vy, &vz,
                                  &ipath, &r.pc, &ppc, &pps, &pmb, &pmo, weighted_run(D) ? &r.w : nullptr);
        else
            ps = o_sphere_sampled(opt, P.n_water, D.pn[pidx], D.pk[pidx], P.wavelength, P.rough_alpha, prad,
                                  P.max_particle_bounces, sgx, sgy, sgz, dscx, dscy, dscz, &x, &y, &z, &vx, &vy, &vz,
                                  &ipath, &r.pc, &ppc, &pps, &pmb, &pmo);
        if (ps == 2) { r.st = 5; res = 1; break; }
        if (ps != 1) { if (COND) atomicAdd(&cstats[8], 1ull); r.pf = ppc ? ppc : OP_OTHER; r.pfs = pps; r.st = 4; res = 1; break; }
        if (COND) { atomicAdd(&cstats[3], 1ull); atomicAdd(&cstats[7], 1ull); }
        apply_moment(D, pidx, vinx, viny, vinz, &vx, &vy, &vz);
        if (weighted_run(D) && roulette(D, r, opt)) res = 1;
    } while (false);
    r.x = x; r.y = y; r.z = z; r.vx = vx; r.vy = vy; r.vz = vz;
    return res;
}

template <class S>
__device__ __forceinline__ bool water_geom(const DevScene& D, Ray& r, S* opt, unsigned long long* cstats, int pidx) {
    const int g = water_geom_visit(D, r, opt, cstats, pidx);
    if (g != 3) return g == 1;
    CondState cs = cond_start();
    return closure_visit(D, r, opt, cstats, pidx, CK_GEOM, &cs, 0) == 1;
}

template <class S>
__device__ __forceinline__ bool water_morph(const DevScene& D, Ray& r, S* opt, unsigned long long* cstats, int pidx) {
    const clr_scene_params& P = D.P;
    float x = r.x, y = r.y, vx = r.vx, vy = r.vy, vz = r.vz;
    const float vinx = vx, viny = vy, vinz = vz;
    const int COND = (P.event_model == 4 || P.event_model == 5);
    bool ended = false;
    do {
        float fr = sqrtf(x * x + y * y);
        float ffx = 1.0f, ffy = 0.0f, ffz = 0.0f;
        if (fr > 1e-12f) { ffx = -y / fr; ffy = x / fr; }
        float ipath = 0.0f;
        int ppc = 0, pps = 0, pmb = 0, pmo = 0;
        int ps = o_spheroid_event(opt, P.n_water, D.pn[pidx], D.pk[pidx], P.wavelength, P.rough_alpha, D.prad[pidx],
                                  P.spheroid_aspect, P.orientation_model, P.orientation_kappa, ffx, ffy, ffz,
                                  P.max_particle_bounces, &vx, &vy, &vz, &ipath, &r.pc, &ppc, &pps, &pmb, &pmo,
                                  weighted_run(D) ? &r.w : nullptr);
        if (ps == 2) { r.st = 5; ended = true; break; }
        if (ps != 1) { if (COND) atomicAdd(&cstats[8], 1ull); r.pf = ppc ? ppc : OP_OTHER; r.pfs = pps; r.st = 4; ended = true; break; }
        if (COND) { atomicAdd(&cstats[5], 1ull); atomicAdd(&cstats[7], 1ull); }
        apply_moment(D, pidx, vinx, viny, vinz, &vx, &vy, &vz);
        if (weighted_run(D) && roulette(D, r, opt)) ended = true;
    } while (false);
    r.vx = vx; r.vy = vy; r.vz = vz;
    return ended;
}

// transmitted through the free surface into the headspace
template <class S>
__device__ __forceinline__ bool water_top(const DevScene& D, Ray& r, S* st) {
    const o_cell C = make_cell(D.P);
    float x = r.x, y = r.y, z = r.z, vx = r.vx, vy = r.vy, vz = r.vz;
    o_bcount bc = {0, 0, 0, 0, 0, 0, 0, 0};
    int hs = 0, hb = 0;
    const int hw = o_headspace(st, &C, &x, &y, &z, &vx, &vy, &vz, &r.ap, &bc, &hs, &hb);
    bool ended = hw != 1;
    if (hw == 1) {}
    else if (hw == 2) r.st = 1;
    else if (hw == 3) r.st = 7;
    else if (hw == 4) r.st = 6;
    else { r.pf = OP_HEADSPACE_NO_BOUNDARY; r.pfs = hs; r.st = 4; }
    add_bounces(r, bc);
    r.x = x; r.y = y; r.z = z; r.vx = vx; r.vy = vy; r.vz = vz;
    return ended;
}

// ---- water iterations that continue inside the acrylic (cell wall or bottom disc) ----
// The traversal of the acrylic solid can take up to 16384 bounces (light trapped by total internal
// reflection); the wavefront engine runs it in bounded pieces, so its loop state travels with the photon.
enum : int { ACR_SIDE = 0, ACR_BOTTOM = 1 };

// Outcome of an iteration once its acrylic traversal (or the bottom-disc entry) gave `where`;
// true when the history ended. The two callers differ only as the reference's branches do.
template <class S>
__device__ __forceinline__ bool acrylic_outcome(const DevScene& D, Ray& r, S* st, int caller, int where, int sub,
                                                float* x, float* y, float* z, float* vx, float* vy, float* vz,
                                                o_bcount* bc) {
    if (where == 1) return false;
    if (where == 2) { r.st = 1; return true; }
    if (where == 3) { r.st = 7; return true; }
    if (where == 5) { r.st = 8; return true; }
    if (where == 4) {
        const o_cell C = make_cell(D.P);
        int hs = 0, hb = 0;
        const int hw = o_headspace(st, &C, x, y, z, vx, vy, vz, &r.ap, bc, &hs, &hb);
        if (hw == 1) return false;
        if (hw == 2) r.st = 1;
        else if (hw == 3) r.st = 7;
        else if (hw == 4) r.st = 6;
        else if (hw == 5 && caller == ACR_SIDE) r.st = 8;
        else { r.pf = OP_HEADSPACE_NO_BOUNDARY; r.pfs = hs; r.st = 4; }
        return true;
    }
    if (caller == ACR_SIDE) r.pf = (sub == OS_ACRYLIC_BOUNCE_LIMIT) ? OP_ACRYLIC_BOUNCE_LIMIT : OP_ACRYLIC_NO_INTERSECTION;
    else r.pf = (sub == OS_ACRYLIC_BOUNCE_LIMIT) ? OP_ACRYLIC_BOUNCE_LIMIT : OP_BOTTOM_GEOMETRY;
    r.pfs = sub;
    r.st = 4;
    return true;
}

// Runs up to `budget` bounces of the traversal (0: to its end). Returns 0 when the iteration ended with
// the photon in the water, 1 when the history ended, 2 when the traversal continues (state in *as).
template <class S>
__device__ __forceinline__ int acrylic_visit(const DevScene& D, Ray& r, S* st, int caller, o_acr_state* as,
                                             int budget) {
    const clr_scene_params& P = D.P;
    const o_cell C = make_cell(P);
    float x = r.x, y = r.y, z = r.z, vx = r.vx, vy = r.vy, vz = r.vz;
    o_bcount bc = {0, 0, 0, 0, 0, 0, 0, 0};
    int sub = 0, nb = 0;
    const int where = o_acrylic_run(st, &C, C.n_air, C.n_bottom_ext, P.zmin, C.Zlow, &x, &y, &z, &vx, &vy, &vz, &r.ap,
                                    &bc, &sub, &nb, as, budget);
    int res = 2;
    if (where >= 0) res = acrylic_outcome(D, r, st, caller, where, sub, &x, &y, &z, &vx, &vy, &vz, &bc) ? 1 : 0;
    add_bounces(r, bc);
    r.x = x; r.y = y; r.z = z; r.vx = vx; r.vy = vy; r.vz = vz;
    return res;
}

// reached the bottom disc: same return codes as acrylic_visit
template <class S>
__device__ __forceinline__ int water_bottom_visit(const DevScene& D, Ray& r, S* st, o_acr_state* as, int budget) {
    const o_cell C = make_cell(D.P);
    float x = r.x, y = r.y, z = r.z, vx = r.vx, vy = r.vy, vz = r.vz;
    o_bcount bc = {0, 0, 0, 0, 0, 0, 0, 0};
    int bs = 0, bb = 0;
    const int e = o_bottom_entry(st, &C, &x, &y, &z, &vx, &vy, &vz, &bc, &bs, &bb);
    int res = 2;
    if (e != 6) res = acrylic_outcome(D, r, st, ACR_BOTTOM, e, bs, &x, &y, &z, &vx, &vy, &vz, &bc) ? 1 : 0;
    add_bounces(r, bc);
    r.x = x; r.y = y; r.z = z; r.vx = vx; r.vy = vy; r.vz = vz;
    if (e != 6) return res;
    *as = o_acr_start();
    return acrylic_visit(D, r, st, ACR_BOTTOM, as, budget);
}

template <class S>
__device__ __forceinline__ bool water_bottom(const DevScene& D, Ray& r, S* st) {
    o_acr_state as;
    return water_bottom_visit(D, r, st, &as, 0) == 1;
}

// transmitted into the acrylic wall
template <class S>
__device__ __forceinline__ bool water_side(const DevScene& D, Ray& r, S* st) {
    o_acr_state as = o_acr_start();
    return acrylic_visit(D, r, st, ACR_SIDE, &as, 0) == 1;
}

// One whole water iteration (flight part and its handler).
template <class S, bool kWeighted>
__device__ __forceinline__ bool water_step(const DevScene& D, Ray& r, S* st, S* opt, unsigned long long* cstats,
                                           uint32_t gid) {
    int pidx = -1;
    const int e = water_flight(D, r, st, opt, cstats, &pidx, gid);
    (void)kWeighted;
    switch (e) {
        case WE_NONE: return false;
        case WE_ENDED: return true;
        case WE_COND: return water_cond(D, r, opt, cstats, pidx);
        case WE_GEOM: return water_geom(D, r, opt, cstats, pidx);
        case WE_MORPH: return water_morph(D, r, opt, cstats, pidx);
        case WE_TOP: return water_top(D, r, st);
        case WE_BOTTOM: return water_bottom(D, r, st);
        default: return water_side(D, r, st);
    }
}

}  // namespace
}  // namespace clr
