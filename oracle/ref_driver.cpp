// ref_driver.cpp -- C entry points over the UNMODIFIED reference sources (kerr.cpp, trajectory.cpp,
// central.cpp, eht.cpp), compiled where they lie by oracle/Makefile into oracle/_ref/libkerr_ref.so.
//
// TEST INFRASTRUCTURE ONLY: used in this container to pin the C restatement (kerr_oracle.c)
// and to generate the golden fixtures under tests/golden/. It builds only where the reference
// tree exists; nothing on the product path loads it.
//
// The ray-level loop (ref_trace_frame) is the reference's own loop shape from
// src/trajectory.cpp:259-392 (photonStepSize -> stepMino -> normalizeAngles ->
// enforceConstraints, thin-disk crossing by linear interpolation, g from circularOmega) driven by
// the scene's tolerance, capture radius and escape radius, through kerr:: calls only.

#include "central.h"
#include "eht.h"
#include "kerr.h"
#include "trajectory.h"

#include "kerr_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

static_assert(sizeof(orc_constants) == sizeof(kerr::Constants), "constants layout");
static_assert(sizeof(orc_state) == sizeof(kerr::State), "state layout");
static_assert(sizeof(orc_derivs) == sizeof(kerr::Derivatives), "derivatives layout");

namespace {

kerr::Constants kc(const orc_constants* c) { return {c->E, c->L, c->Q, c->mu}; }
kerr::State ks(const orc_state* s) { return {s->t, s->r, s->theta, s->phi, s->vr, s->vtheta}; }
void put(const kerr::Constants& c, orc_constants* o) { *o = {c.E, c.L, c.Q, c.mu}; }
void put(const kerr::State& s, orc_state* o) { *o = {s.t, s.r, s.theta, s.phi, s.vr, s.vtheta}; }

kerr::Frame zamo_frame(double a, double r, double th) {
    return kerr::observerFrame(a, r, th, kerr::zamoFourVelocity(a, r, th));
}

void pinhole(const orc_scene* sc, double alpha, double beta, kerr::Constants& c, kerr::State& s) {
    const kerr::Frame f = zamo_frame(sc->a, sc->r_obs, sc->theta_obs);
    const double lr = -1.0, lt = -beta / sc->r_obs, lp = alpha / sc->r_obs;
    const double n = std::sqrt(lr * lr + lt * lt + lp * lp);
    const double look[3] = {lr / n, lt / n, lp / n};
    kerr::photonFromFrame(sc->a, sc->r_obs, sc->theta_obs, sc->phi_obs, f, look, c, s);
}

void sky(double a, const kerr::Constants& c, const kerr::State& x, double* th, double* ph) {
    const kerr::Derivatives d = kerr::derivatives(a, c, x);
    auto v = kerr::cartesianVelocity(a, x.r, x.theta, x.phi, x.vr, x.vtheta, d.dphi);
    const double n = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    *th = std::acos(std::clamp(-v[2] / n, -1.0, 1.0));
    *ph = std::atan2(-v[1] / n, -v[0] / n);
}

void ray_clear(orc_ray* out) {
    std::memset(out, 0, sizeof(*out));
    out->r_disk = out->phi_disk = out->g = out->theta_inf = out->phi_inf = NAN;
}

// The reference loop shape from a launched photon.
void trace_launched(const orc_scene* sc, kerr::Constants c, kerr::State s, orc_ray* out) {
    out->E = c.E, out->L = c.L, out->Q = c.Q;
    const double a = sc->a;
    const bool naked = std::abs(a) > 1.0;
    const double rcap = kerr::horizonRadius(a) * (1.0 + sc->capture_eps);
    const double resc = std::max(sc->r_escape, 1.5 * sc->r_obs);
    const double rin = sc->r_disk_in > 0.0 ? sc->r_disk_in : kerr::iscoRadius(a, true);
    const double hp = 0.5 * kerr::kPi;
    for (int i = 0; i < sc->max_steps; ++i) {
        const kerr::State prev = s;
        kerr::stepMino(a, c, s, -kerr::photonStepSize(a, c, s, sc->tol));
        kerr::normalizeAngles(s);
        kerr::enforceConstraints(a, c, s);
        out->steps = i + 1;
        if (!std::isfinite(s.r)) return;
        if ((prev.theta - hp) * (s.theta - hp) < 0.0) {
            const double f = (prev.theta - hp) / (prev.theta - s.theta);
            const double rc = prev.r + f * (s.r - prev.r);
            if (rc >= rin && rc <= sc->r_disk_out) {
                const double w = kerr::circularOmega(a, rc, true);
                const double gtt = -(1.0 - 2.0 / rc), gtp = -2.0 * a / rc, gpp = rc * rc + a * a + 2.0 * a * a / rc;
                const double norm = -(gtt + 2.0 * gtp * w + gpp * w * w);
                if (norm > 0.0) {
                    out->outcome = ORC_DISK;
                    out->r_disk = rc;
                    double ph = prev.phi + f * (s.phi - prev.phi);
                    ph -= 2.0 * kerr::kPi * std::floor(ph / (2.0 * kerr::kPi));
                    out->phi_disk = ph;
                    out->g = std::sqrt(norm) / (c.E - c.L * w);
                    return;
                }
            }
        }
        // Past a = 1 there is no horizon: the renderer's rules (shaders/trace.frag:1772-1787) -- the
        // ring singularity where Sigma < 4e-4, and the sky of the r < 0 region beyond r = -resc.
        if (naked) {
            const double cs = std::cos(s.theta);
            if (s.r * s.r + a * a * cs * cs < 4e-4) {
                out->outcome = ORC_RING;
                return;
            }
        } else if (s.r < rcap && s.r < prev.r) {
            out->outcome = ORC_CAPTURED;
            return;
        }
        const bool far = naked && s.r < -resc && s.r < prev.r;
        if ((s.r > resc && s.r > prev.r) || far) {
            const double target = far ? -resc : resc;
            kerr::State x = s;
            if (std::abs(s.theta - prev.theta) < 1.0) {
                const double f = (target - prev.r) / (s.r - prev.r);
                x.r = target;
                x.theta = prev.theta + f * (s.theta - prev.theta);
                x.phi = prev.phi + f * (s.phi - prev.phi);
                x.vr = prev.vr + f * (s.vr - prev.vr);
                x.vtheta = prev.vtheta + f * (s.vtheta - prev.vtheta);
            }
            out->outcome = far ? ORC_ESCAPED_BEYOND : ORC_ESCAPED;
            sky(a, c, x, &out->theta_inf, &out->phi_inf);
            return;
        }
    }
}

void trace_one(const orc_scene* sc, double alpha, double beta, orc_ray* out) {
    ray_clear(out);
    kerr::Constants c;
    kerr::State s;
    pinhole(sc, alpha, beta, c, s);
    trace_launched(sc, c, s, out);
}

}  // namespace

extern "C" {

void ref_derivatives(double a, const orc_constants* c, const orc_state* s, orc_derivs* d) {
    const kerr::Derivatives r = kerr::derivatives(a, kc(c), ks(s));
    *d = {r.dt, r.dr, r.dtheta, r.dphi, r.dvr, r.dvtheta};
}
void ref_step_mino(double a, const orc_constants* c, orc_state* s, double h) {
    kerr::State x = ks(s);
    kerr::stepMino(a, kc(c), x, h);
    put(x, s);
}
double ref_photon_step_size(double a, const orc_constants* c, const orc_state* s, double tol) {
    return kerr::photonStepSize(a, kc(c), ks(s), tol);
}
void ref_enforce_constraints(double a, const orc_constants* c, orc_state* s) {
    kerr::State x = ks(s);
    kerr::enforceConstraints(a, kc(c), x);
    put(x, s);
}
void ref_normalize_angles(orc_state* s) {
    kerr::State x = ks(s);
    kerr::normalizeAngles(x);
    put(x, s);
}
double ref_radial_potential(double a, const orc_constants* c, double r) { return kerr::radialPotential(a, kc(c), r); }
double ref_polar_potential(double a, const orc_constants* c, double th) { return kerr::polarPotential(a, kc(c), th); }
double ref_inflow_factor(double P, double vr, double delta, double K) { return kerr::inflowFactor(P, vr, delta, K); }
double ref_horizon_radius(double a) { return kerr::horizonRadius(a); }
double ref_isco_radius(double a, int prograde) { return kerr::iscoRadius(a, prograde != 0); }
double ref_photon_orbit_radius(double a, int prograde) { return kerr::photonOrbitRadius(a, prograde != 0); }
double ref_circular_omega(double a, double r, int prograde) { return kerr::circularOmega(a, r, prograde != 0); }
void ref_launch_from_zamo(double a, double r, double th, double ph, const double v[3], double mu, orc_constants* c,
                          orc_state* s) {
    kerr::Constants x;
    kerr::State y;
    kerr::launchFromZamo(a, r, th, ph, v, mu, x, y);
    put(x, c);
    put(y, s);
}
void ref_zamo_four_velocity(double a, double r, double th, double u[4]) {
    const kerr::Vec4 v = kerr::zamoFourVelocity(a, r, th);
    for (int i = 0; i < 4; ++i) u[i] = v[i];
}
void ref_observer_frame(double a, double r, double th, const double u[4], orc_frame* f) {
    const kerr::Frame fr = kerr::observerFrame(a, r, th, {u[0], u[1], u[2], u[3]});
    for (int k = 0; k < 4; ++k)
        for (int i = 0; i < 4; ++i) f->e[k][i] = fr.e[k][i];
}
void ref_photon_from_frame(double a, double r, double th, double ph, const orc_frame* f, const double look[3],
                           orc_constants* c, orc_state* s) {
    kerr::Frame fr;
    for (int k = 0; k < 4; ++k)
        for (int i = 0; i < 4; ++i) fr.e[k][i] = f->e[k][i];
    kerr::Constants x;
    kerr::State y;
    kerr::photonFromFrame(a, r, th, ph, fr, look, x, y);
    put(x, c);
    put(y, s);
}
void ref_cartesian_velocity(double a, double r, double th, double ph, double dr, double dth, double dph, double o[3]) {
    auto v = kerr::cartesianVelocity(a, r, th, ph, dr, dth, dph);
    o[0] = v[0], o[1] = v[1], o[2] = v[2];
}
int ref_critical_curve(double a, double incl, int samples, double* alpha, double* beta, int cap) {
    const std::vector<eht::Point> c = eht::criticalCurve(a, incl, samples);
    const int n = std::min<int>(cap, static_cast<int>(c.size()));
    for (int k = 0; k < n; ++k) alpha[k] = c[k].alpha, beta[k] = c[k].beta;
    return n;
}
double ref_critical_radius(const double* alpha, const double* beta, int n, double psi) {
    std::vector<eht::Point> c(n);
    for (int k = 0; k < n; ++k) c[k] = {alpha[k], beta[k]};
    return eht::criticalRadius(c, psi);
}
int ref_eht_captured(double a, double incl, double alpha, double beta) {
    eht::View v;
    v.a = a;
    v.inclination = incl;
    return eht::traceRay(v, eht::Flow{}, alpha, beta, false).captured ? 1 : 0;
}
double ref_bending_angle(double R, double alpha) { return central::bendingAngle(R, alpha); }

// The reference's own trajectory::traceRay (tolerance 0.01, horizon r_+ + 0.01, escape
// max(escapeRadius, 1.5 r)) from a ZAMO at (a, r, theta, phi). Returns the RayEnd code.
int ref_trajectory_trace(double a, double r, double th, double ph, const double look[3], int disk, double r_in,
                         double r_out, double escape, double out[9]) {
    trajectory::RayScene scene;
    scene.disk = disk != 0;
    scene.diskInner = r_in;
    scene.diskOuter = r_out;
    scene.escapeRadius = escape;
    const trajectory::RayReport rep = trajectory::traceRay(a, r, th, ph, zamo_frame(a, r, th), look, scene);
    out[0] = rep.rEnd, out[1] = rep.g, out[2] = rep.skyDirection[0], out[3] = rep.skyDirection[1];
    out[4] = rep.skyDirection[2], out[5] = rep.rMin, out[6] = rep.turns, out[7] = rep.energy, out[8] = rep.delay;
    return static_cast<int>(rep.end);
}

// trajectory::traceRay with an arbitrary camera frame (16 doubles, e[k][i]): moving cameras and
// cameras inside the horizon. out[] as ref_trajectory_trace.
int ref_trajectory_trace_framed(double a, double r, double th, double ph, const double* frame16,
                                const double look[3], int disk, double r_in, double r_out, double escape,
                                double out[9]) {
    trajectory::RayScene scene;
    scene.disk = disk != 0;
    scene.diskInner = r_in;
    scene.diskOuter = r_out;
    scene.escapeRadius = escape;
    kerr::Frame f;
    for (int k = 0; k < 4; ++k)
        for (int i = 0; i < 4; ++i) f.e[k][i] = frame16[4 * k + i];
    const trajectory::RayReport rep = trajectory::traceRay(a, r, th, ph, f, look, scene);
    out[0] = rep.rEnd, out[1] = rep.g, out[2] = rep.skyDirection[0], out[3] = rep.skyDirection[1];
    out[4] = rep.skyDirection[2], out[5] = rep.rMin, out[6] = rep.turns, out[7] = rep.energy, out[8] = rep.delay;
    return static_cast<int>(rep.end);
}

// eht::render (src/eht.cpp:321-347) of View{a, inclination, halfWidth, size, frequency, massSolar}
// and Flow{n0, T0, beta, keplerian, height, sinThetaB}: intensity and shadow, row-major.
void ref_eht_render(double a, double inclination, double half_width, int size, double frequency, double mass_solar,
                    const double* flow6, int threads, double* intensity, unsigned char* shadow) {
    eht::View v;
    v.a = a, v.inclination = inclination, v.halfWidth = half_width, v.size = size, v.frequency = frequency;
    v.massSolar = mass_solar;
    eht::Flow f;
    f.n0 = flow6[0], f.T0 = flow6[1], f.beta = flow6[2], f.keplerian = flow6[3], f.height = flow6[4];
    f.sinThetaB = flow6[5];
    const eht::Image img = eht::render(v, f, threads);
    for (size_t k = 0; k < img.intensity.size(); ++k) {
        intensity[k] = img.intensity[k];
        shadow[k] = img.shadow[k];
    }
}

double ref_eht_calibrate(double a, double inclination, double half_width, int size, double frequency, double mass_solar,
                         const double* flow6, double target_jy, double theta_g_uas, int threads) {
    eht::View v;
    v.a = a, v.inclination = inclination, v.halfWidth = half_width, v.size = size, v.frequency = frequency;
    v.massSolar = mass_solar;
    eht::Flow f;
    f.n0 = flow6[0], f.T0 = flow6[1], f.beta = flow6[2], f.keplerian = flow6[3], f.height = flow6[4];
    f.sinThetaB = flow6[5];
    return eht::calibrate(v, f, target_jy, theta_g_uas, threads);
}

// trajectory::predict (src/trajectory.cpp:130-185) of one particle: scalars into out[7] (fate,
// duration, rMin, rMax, periapses, precessionDeg, number of points) and up to cap points (x, y, z).
void ref_predict(double a, const orc_constants* c, const orc_state* s, double max_time, double min_spacing,
                 int max_points, double surface, double escape_radius, double out[7], double* points, int cap) {
    const trajectory::Path p = trajectory::predict(a, kc(c), ks(s), max_time, min_spacing,
                                                   static_cast<size_t>(max_points), surface, escape_radius);
    out[0] = static_cast<double>(static_cast<int>(p.fate));
    out[1] = p.duration, out[2] = p.rMin, out[3] = p.rMax, out[4] = p.periapses, out[5] = p.precessionDeg;
    out[6] = static_cast<double>(p.points.size());
    for (size_t k = 0; k < p.points.size() && static_cast<int>(k) < cap; ++k)
        for (int j = 0; j < 3; ++j) points[3 * k + j] = p.points[k][j];
}

double ref_eht_angular_scale(double mass_solar, double distance_pc) { return eht::angularScale(mass_solar, distance_pc); }

double ref_eht_flux(const double* intensity, int size, double half_width, double theta_g_uas) {
    eht::Image img;
    img.size = size;
    img.halfWidth = half_width;
    img.intensity.assign(intensity, intensity + static_cast<size_t>(size) * size);
    return eht::flux(img, theta_g_uas);
}

void ref_trace_ray(const orc_scene* sc, double alpha, double beta, orc_ray* out) { trace_one(sc, alpha, beta, out); }

// The same loop for a camera with any frame (16 doubles e[k][i]) at the scene's position, with
// trajectory::traceRay's inside-horizon rule (src/trajectory.cpp:236-244).
void ref_trace_framed(const orc_scene* sc, const double* frame16, const double look[3], orc_ray* out) {
    ray_clear(out);
    kerr::Frame f;
    for (int k = 0; k < 4; ++k)
        for (int i = 0; i < 4; ++i) f.e[k][i] = frame16[4 * k + i];
    kerr::Constants c;
    kerr::State s;
    kerr::photonFromFrame(sc->a, sc->r_obs, sc->theta_obs, sc->phi_obs, f, look, c, s);
    const double rh = kerr::horizonRadius(sc->a);
    if (sc->r_obs < rh && 2.0 * rh * c.E - sc->a * c.L < 0.0) {
        out->E = c.E, out->L = c.L, out->Q = c.Q;
        out->outcome = ORC_CAPTURED;
        return;
    }
    trace_launched(sc, c, s, out);
}

// Whole frame on nthreads std::threads with an atomic row counter (src/eht.cpp:321-347).
void ref_trace_frame(const orc_scene* sc, int w, int h, double alo, double ahi, double blo, double bhi, int nthreads,
                     int32_t* outcome, double* r_disk, double* phi_disk, double* g, double* th_inf, double* ph_inf,
                     int32_t* steps) {
    std::atomic<int> next_row{0};
    auto work = [&]() {
        for (int row = next_row++; row < h; row = next_row++) {
            const double beta = bhi - (row + 0.5) * (bhi - blo) / h;
            for (int col = 0; col < w; ++col) {
                const double alpha = alo + (col + 0.5) * (ahi - alo) / w;
                orc_ray ray;
                trace_one(sc, alpha, beta, &ray);
                const size_t k = static_cast<size_t>(row) * w + col;
                if (outcome) outcome[k] = ray.outcome;
                if (r_disk) r_disk[k] = ray.r_disk;
                if (phi_disk) phi_disk[k] = ray.phi_disk;
                if (g) g[k] = ray.g;
                if (th_inf) th_inf[k] = ray.theta_inf;
                if (ph_inf) ph_inf[k] = ray.phi_inf;
                if (steps) steps[k] = ray.steps;
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < std::max(nthreads, 1); ++t) pool.emplace_back(work);
    work();
    for (std::thread& t : pool) t.join();
}

}  // extern "C"
