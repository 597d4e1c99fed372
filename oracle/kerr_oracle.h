/*
 * kerr_oracle.h -- CPU restatement of the reference's Kerr photon path, in plain C.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker for the CUDA tracer in
 * black_simulation_gb300/csrc. Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline / reference legs may load it. The product path never calls it.
 *
 * Parity status: pinned. Every per-step function is compared with the reference
 * compiled from its own sources (oracle/Makefile -> oracle/_ref/libkerr_ref.so) and with
 * golden vectors generated from it (tests/golden/make_golden.py).
 *
 * Units: G = c = M = 1. Coordinates: ingoing Kerr-Schild (t, r, theta, phi), Mino time.
 * Reference files cited as path:line inside the Black_simulation project.
 */
#ifndef KERR_ORACLE_H
#define KERR_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { double E, L, Q, mu; } orc_constants;            /* src/kerr.h:81-86 */
typedef struct { double t, r, theta, phi, vr, vtheta; } orc_state; /* src/kerr.h:91-95 */
typedef struct { double dt, dr, dtheta, dphi, dvr, dvtheta; } orc_derivs; /* src/kerr.h:97-99 */
typedef struct { double e[4][4]; } orc_frame;                    /* src/kerr.h:143-145, e[k][mu] */

/* ---- radii and metric (src/kerr.cpp:157-299) ---- */
double orc_horizon_radius(double a);
double orc_isco_radius(double a, int prograde);
double orc_photon_orbit_radius(double a, int prograde);
double orc_circular_omega(double a, double r, int prograde);
void orc_metric_tensor(double a, double r, double theta, double g[4][4]);

/* ---- geodesic primitives (src/kerr.cpp:323-604) ---- */
double orc_inflow_factor(double P, double vr, double delta, double K);
void orc_derivatives(double a, const orc_constants* c, const orc_state* s, orc_derivs* d);
double orc_radial_potential(double a, const orc_constants* c, double r);
double orc_polar_potential(double a, const orc_constants* c, double theta);
void orc_launch_from_zamo(double a, double r, double theta, double phi, const double v[3], double mu,
                          orc_constants* c, orc_state* s);
void orc_zamo_four_velocity(double a, double r, double theta, double u[4]);
void orc_observer_frame(double a, double r, double theta, const double u[4], orc_frame* f);
void orc_photon_from_frame(double a, double r, double theta, double phi, const orc_frame* f,
                           const double look[3], orc_constants* c, orc_state* s);
void orc_step_mino(double a, const orc_constants* c, orc_state* s, double h);
void orc_enforce_constraints(double a, const orc_constants* c, orc_state* s);
double orc_photon_step_size(double a, const orc_constants* c, const orc_state* s, double tol);
void orc_normalize_angles(orc_state* s);
void orc_to_cartesian(double a, double r, double theta, double phi, double out[3]);
void orc_cartesian_velocity(double a, double r, double theta, double phi, double dr, double dtheta,
                            double dphi, double out[3]);

/* ---- analytic shadow (src/eht.cpp:52-97) ---- */
int orc_critical_curve(double a, double inclination, int samples, double* alpha, double* beta, int cap);
double orc_critical_radius(const double* alpha, const double* beta, int n, double psi);
/* The critical curve as a pinhole camera at finite r_obs sees it (image-plane units M at r_obs). */
int orc_critical_curve_finite(double a, double r_obs, double theta_obs, int samples, double* alpha,
                              double* beta, int cap);

/* ---- ray-level tracer ---- */
/* Past a = 1 (no horizon; shaders/trace.frag:1552-1554, 1768-1787): no capture; a ray whose Sigma
 * falls below 4e-4 has struck the ring singularity (ORC_RING), and one that passed through the
 * ring's disk and leaves below r = -max(r_escape, 1.5 r_obs) escaped to the sky of the r < 0
 * region (ORC_ESCAPED_BEYOND, with its direction like ORC_ESCAPED). */
enum { ORC_UNFINISHED = 0, ORC_CAPTURED = 1, ORC_DISK = 2, ORC_ESCAPED = 3, ORC_ESCAPED_BEYOND = 4, ORC_RING = 5 };
enum { ORC_METHOD_RK4 = 0, ORC_METHOD_DP5 = 1 };

typedef struct {
    double a, r_obs, theta_obs, phi_obs;
    double r_disk_in, r_disk_out;  /* r_disk_in <= 0: prograde ISCO */
    double r_escape;               /* escaped once r > max(r_escape, 1.5 r_obs) while rising */
    double capture_eps;            /* captured once r < r_+ (1 + capture_eps) while falling */
    double tol;                    /* RK4: photonStepSize tolerance; DP5: rtol = atol */
    int max_steps;
    int method;
} orc_scene;

typedef struct {
    int32_t outcome, steps, rejected, pad;
    double r_disk, phi_disk, g, theta_inf, phi_inf;
    double E, L, Q;
} orc_ray;

/* Launches the photon a ZAMO pinhole camera sees at image-plane point (alpha, beta). */
void orc_pinhole_launch(const orc_scene* sc, double alpha, double beta, orc_constants* c, orc_state* s);
void orc_trace_ray(const orc_scene* sc, double alpha, double beta, orc_ray* out);
/* Whole frame, pixel centres, row-major from the top (src/eht.cpp:321-347 layout); nthreads workers
 * pull rows from an atomic counter. Outputs are SoA arrays of w*h entries (any may be NULL). */
void orc_trace_frame(const orc_scene* sc, int width, int height, double alpha_lo, double alpha_hi,
                     double beta_lo, double beta_hi, int nthreads, int32_t* outcome, double* r_disk,
                     double* phi_disk, double* g, double* theta_inf, double* phi_inf, int32_t* steps);
/* Per-ray variant: explicit arrays, n rays, shared scene except (a, r_obs, theta_obs) per ray. */
void orc_trace_rays(const orc_scene* sc, int64_t n, const double* a, const double* r_obs,
                    const double* theta_obs, const double* alpha, const double* beta, int nthreads,
                    int32_t* outcome, double* r_disk, double* phi_disk, double* g, double* theta_inf,
                    double* phi_inf, int32_t* steps);

/* A camera at (sc->r_obs, sc->theta_obs, sc->phi_obs) with any frame (moving; inside the horizon
 * too) and a look direction on its (r, theta, phi) axes: trajectory::traceRay's launch and its
 * inside-horizon rule (src/trajectory.cpp:214-247), then the scene's tracer. */
void orc_trace_framed(const orc_scene* sc, const orc_frame* f, const double look[3], orc_ray* out);

/* Capture test used by the DP5 tracer near the horizon: 1 if R(r') > 0 on [r_+(1+eps), r]. */
int orc_no_radial_root_below(double a, double E, double L, double Q, double r, double eps);

#ifdef __cplusplus
}
#endif
#endif
