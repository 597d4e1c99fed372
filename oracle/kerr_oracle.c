/*
 * kerr_oracle.c -- CPU restatement (FP64, plain C) of the reference's photon path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA tracer, never the product.
 *
 * Two ray-level integrators live here:
 *   ORC_METHOD_RK4  the reference's own loop shape: photonStepSize -> stepMino ->
 *                   normalizeAngles -> enforceConstraints (src/trajectory.cpp:259-262), with the
 *                   thin-disk rule and g of src/trajectory.cpp:305-324.
 *   ORC_METHOD_DP5  the adaptive Dormand-Prince 5(4) tracer with dense-output event location
 *                   that the CUDA FP64 kernel implements step for step. It is checked against
 *                   RK4 at tolerance 1e-4 (error ~1e-8 by Richardson) in the tests.
 * Built with -O2 -ffp-contract=off so x86 and Arm give the same bits.
 */
#include "kerr_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>

#define ORC_PI 3.14159265358979323846

static double dmax(double x, double y) { return x > y ? x : y; }
static double dmin(double x, double y) { return x < y ? x : y; }
static double dclamp(double x, double lo, double hi) { return x < lo ? lo : (x > hi ? hi : x); }
static int is_naked(double a) { return fabs(a) > 1.0; }

/* ---------------------------------------------------------------- radii ---- */

/* r_+ = 1 + sqrt(1 - a^2); 0 past a = 1 (src/kerr.cpp:157-160). */
double orc_horizon_radius(double a) {
    if (is_naked(a)) return 0.0;
    return 1.0 + sqrt(dmax(0.0, 1.0 - a * a));
}

/* Energy per unit mass of the circular equatorial orbit at r (Bardeen, Press & Teukolsky 1972), 1e30
 * where there is none (src/kerr.cpp:122-129). */
static double circular_energy(double a, double r, int prograde) {
    const double sg = prograde ? 1.0 : -1.0, q = sqrt(r);
    const double den = r * q - 3.0 * q + 2.0 * sg * a;
    if (den <= 0.0) return 1e30;
    return (r * q - 2.0 * q + sg * a) / (pow(r, 0.75) * sqrt(den));
}

/* The radius of least circular-orbit energy in [lo, hi]: the best of 4001 points of a geometric
 * grid, then 80 golden-section steps between its neighbours (src/kerr.cpp:131-153). */
static double least_energy_radius(double a, int prograde, double lo, double hi) {
    const int n = 4000;
    int best = 0;
    double best_e = 1e30;
    for (int k = 0; k <= n; ++k) {
        const double e = circular_energy(a, lo * pow(hi / lo, (double)k / n), prograde);
        if (e < best_e) {
            best_e = e;
            best = k;
        }
    }
    double x0 = lo * pow(hi / lo, (best > 1 ? best - 1 : 0) / (double)n);
    double x1 = lo * pow(hi / lo, (best + 1 < n ? best + 1 : n) / (double)n);
    const double gr = 0.5 * (sqrt(5.0) - 1.0);
    for (int k = 0; k < 80; ++k) {
        const double u = x1 - gr * (x1 - x0), v = x0 + gr * (x1 - x0);
        if (circular_energy(a, u, prograde) < circular_energy(a, v, prograde)) x1 = v;
        else x0 = u;
    }
    return 0.5 * (x0 + x1);
}

/* ISCO: Bardeen-Press-Teukolsky (src/kerr.cpp:179-190); past a = 1 the least-energy search, prograde
 * over [1e-3, 30], retrograde from just outside the retrograde photon orbit to 60 (src/kerr.cpp:180-185). */
double orc_isco_radius(double a, int prograde) {
    if (is_naked(a))
        return prograde ? least_energy_radius(a, 1, 1e-3, 30.0)
                        : least_energy_radius(a, 0, orc_photon_orbit_radius(a, 0) * 1.0001, 60.0);
    const double z1 = 1.0 + cbrt(1.0 - a * a) * (cbrt(1.0 + a) + cbrt(1.0 - a));
    const double z2 = sqrt(3.0 * a * a + z1 * z1);
    const double w = sqrt(dmax(0.0, (3.0 - z1) * (3.0 + z1 + 2.0 * z2)));
    return prograde ? 3.0 + z2 - w : 3.0 + z2 + w;
}

/* Circular equatorial photon orbit 2 (1 + cos(2/3 acos(-+a))) (src/kerr.cpp:192-206). */
double orc_photon_orbit_radius(double a, int prograde) {
    if (is_naked(a)) {
        if (prograde) return 0.0;
        double lo = 3.0, hi = 3.0 + 2.0 * fabs(a);
        for (int k = 0; k < 100; ++k) {
            const double m = 0.5 * (lo + hi);
            if (m * (m - 3.0) * (m - 3.0) < 4.0 * a * a) lo = m; else hi = m;
        }
        return 0.5 * (lo + hi);
    }
    const double sgn = prograde ? -1.0 : 1.0;
    return 2.0 * (1.0 + cos(2.0 / 3.0 * acos(sgn * a)));
}

/* Keplerian d(phi)/dt of a circular equatorial orbit (src/kerr.cpp:296-299). */
double orc_circular_omega(double a, double r, int prograde) {
    const double sgn = prograde ? 1.0 : -1.0;
    return sgn / (r * sqrt(r) + sgn * a);
}

/* Covariant Kerr-Schild metric (src/kerr.cpp:238-254). */
void orc_metric_tensor(double a, double r, double theta, double g[4][4]) {
    const double sn = sin(theta), cs = cos(theta), sn2 = sn * sn;
    const double sigma = r * r + a * a * cs * cs;
    const double rra = r * r + a * a;
    const double A = rra * rra - a * a * (r * r - 2.0 * r + a * a) * sn2;
    const double f = 2.0 * r / sigma;
    memset(g, 0, sizeof(double) * 16);
    g[0][0] = -(1.0 - f);
    g[0][1] = g[1][0] = f;
    g[0][3] = g[3][0] = -f * a * sn2;
    g[1][1] = 1.0 + f;
    g[1][3] = g[3][1] = -a * sn2 * (1.0 + f);
    g[2][2] = sigma;
    g[3][3] = A * sn2 / sigma;
}

static double metric_dot(double g[4][4], const double* x, const double* y) {
    double acc = 0.0;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) acc += g[i][j] * x[i] * y[j];
    return acc;
}

/* ------------------------------------------------------- geodesic core ---- */

/* (P + vr) / Delta without the horizon's 0/0: K / (P - vr) when P and vr have opposite signs
 * (src/kerr.cpp:323-329). */
double orc_inflow_factor(double P, double vr, double delta, double K) {
    if (P * vr < 0.0) return K / (P - vr);
    const double d = fabs(delta) > 1e-12 ? delta : copysign(1e-12, delta);
    return (P + vr) / d;
}

/* sin^3 keeping its sign, bounded away from 0 (src/kerr.cpp:11-14). */
static double signed_sin_cubed(double s) {
    const double m = dmax(fabs(s), 1e-9);
    return (s < 0.0 ? -m : m) * m * m;
}

/* Second-order Carter system in Mino time (src/kerr.cpp:331-351). */
void orc_derivatives(double a, const orc_constants* c, const orc_state* s, orc_derivs* d) {
    const double r = s->r;
    const double sn = sin(s->theta), cs = cos(s->theta);
    const double sn2 = dmax(sn * sn, 1e-18);
    const double a2 = a * a, mu2 = c->mu * c->mu;
    const double delta = r * r - 2.0 * r + a2;
    const double rra = r * r + a2;
    const double P = c->E * rra - a * c->L;
    const double x = c->L - a * c->E;
    const double K = mu2 * r * r + x * x + c->Q;
    const double inflow = orc_inflow_factor(P, s->vr, delta, K);
    d->dr = s->vr;
    d->dtheta = s->vtheta;
    d->dvr = 2.0 * c->E * r * P - (r - 1.0) * K - delta * mu2 * r;
    d->dvtheta = sn * cs * a2 * (mu2 - c->E * c->E) + c->L * c->L * cs / signed_sin_cubed(sn);
    d->dphi = a * inflow - a * c->E + c->L / sn2;
    d->dt = rra * inflow - a * (a * c->E * sn * sn - c->L) - s->vr;
}

/* R(r) = P^2 - Delta K (src/kerr.cpp:353-358). */
double orc_radial_potential(double a, const orc_constants* c, double r) {
    const double delta = r * r - 2.0 * r + a * a;
    const double P = c->E * (r * r + a * a) - a * c->L;
    const double x = c->L - a * c->E;
    return P * P - delta * (c->mu * c->mu * r * r + x * x + c->Q);
}

/* Theta(theta) (src/kerr.cpp:360-363). */
double orc_polar_potential(double a, const orc_constants* c, double theta) {
    const double sn = sin(theta), cs = cos(theta);
    return c->Q - cs * cs * (a * a * (c->mu * c->mu - c->E * c->E) + c->L * c->L / dmax(sn * sn, 1e-18));
}

typedef struct { double sigma, delta, A, omega; } orc_metric;

/* Sigma, Delta, A, frame-dragging omega (src/kerr.cpp:227-236). */
static orc_metric metric_at(double a, double r, double theta) {
    const double sn = sin(theta), cs = cos(theta);
    orc_metric m;
    m.sigma = r * r + a * a * cs * cs;
    m.delta = r * r - 2.0 * r + a * a;
    const double rra = r * r + a * a;
    m.A = rra * rra - a * a * m.delta * sn * sn;
    m.omega = 2.0 * a * r / m.A;
    return m;
}

/* Launch from a ZAMO with velocity v on its (r, theta, phi) axes (src/kerr.cpp:365-407). */
void orc_launch_from_zamo(double a, double r, double theta, double phi, const double v[3], double mu,
                          orc_constants* c, orc_state* s) {
    const orc_metric m = metric_at(a, r, theta);
    const double sn = sin(theta), cs = cos(theta);
    double gamma = 1.0;
    if (mu > 0.0) {
        const double v2 = dmin(v[0] * v[0] + v[1] * v[1] + v[2] * v[2], 1.0 - 1e-12);
        gamma = 1.0 / sqrt(1.0 - v2);
    }
    c->mu = mu;
    c->L = gamma * v[2] * sqrt(m.A / m.sigma) * sn;
    c->E = gamma * sqrt(m.sigma * m.delta / m.A) + m.omega * c->L;
    s->t = 0.0;
    s->r = r;
    s->theta = theta;
    s->phi = phi;
    s->vr = gamma * v[0] * sqrt(m.sigma * m.delta);
    s->vtheta = gamma * v[1] * sqrt(m.sigma);
    if (mu == 0.0) {
        const double inv = 1.0 / c->E;
        c->E = 1.0;
        c->L *= inv;
        s->vr *= inv;
        s->vtheta *= inv;
    }
    c->Q = s->vtheta * s->vtheta + cs * cs * (a * a * (mu * mu - c->E * c->E) + c->L * c->L / dmax(sn * sn, 1e-18));
    if (mu == 0.0 && fabs(c->L) < 3e-4 * sqrt(dmax(c->Q + a * a, 0.0))) {
        c->L = 0.0;
        c->Q = s->vtheta * s->vtheta - cs * cs * a * a;
    }
}

/* u = (e_t + omega e_phi) / alpha (src/kerr.cpp:424-430). */
void orc_zamo_four_velocity(double a, double r, double theta, double u[4]) {
    const orc_metric m = metric_at(a, r, theta);
    const double ut = sqrt(m.A / (m.sigma * m.delta));
    u[0] = ut;
    u[1] = 0.0;
    u[2] = 0.0;
    u[3] = m.omega * ut;
}

/* Gram-Schmidt from u through the theta, phi, r coordinate directions (src/kerr.cpp:432-456). */
void orc_observer_frame(double a, double r, double theta, const double u[4], orc_frame* f) {
    double g[4][4];
    orc_metric_tensor(a, r, theta, g);
    memcpy(f->e[0], u, sizeof(double) * 4);
    static const int coord[3] = {2, 3, 1};  /* direction tried, and the slot it fills */
    for (int k = 0; k < 3; ++k) {
        double w[4] = {0.0, 0.0, 0.0, 0.0};
        w[coord[k]] = 1.0;
        const double along = metric_dot(g, w, u);
        for (int i = 0; i < 4; ++i) w[i] += along * u[i];
        for (int j = 0; j < k; ++j) {
            const double* e = f->e[coord[j]];
            const double p = metric_dot(g, w, e);
            for (int i = 0; i < 4; ++i) w[i] -= p * e[i];
        }
        const double n = sqrt(dmax(metric_dot(g, w, w), 1e-300));
        for (int i = 0; i < 4; ++i) f->e[coord[k]][i] = w[i] / n;
    }
}

/* The photon arriving along -look with unit energy in the frame, plus the axis snap
 * (src/kerr.cpp:458-483, src/kerr.h:115). */
void orc_photon_from_frame(double a, double r, double theta, double phi, const orc_frame* f,
                           const double look[3], orc_constants* c, orc_state* s) {
    double p[4], low[4], g[4][4];
    for (int i = 0; i < 4; ++i)
        p[i] = f->e[0][i] - look[0] * f->e[1][i] - look[1] * f->e[2][i] - look[2] * f->e[3][i];
    orc_metric_tensor(a, r, theta, g);
    for (int i = 0; i < 4; ++i) {
        low[i] = 0.0;
        for (int j = 0; j < 4; ++j) low[i] += g[i][j] * p[j];
    }
    const double sigma = metric_at(a, r, theta).sigma;
    const double sn = sin(theta), cs = cos(theta);
    c->mu = 0.0;
    c->E = -low[0];
    c->L = low[3];
    s->t = 0.0;
    s->r = r;
    s->theta = theta;
    s->phi = phi;
    s->vr = sigma * p[1];
    s->vtheta = low[2];
    c->Q = s->vtheta * s->vtheta + cs * cs * (c->L * c->L / dmax(sn * sn, 1e-18) - a * a * c->E * c->E);
    if (fabs(c->L) < 3e-4 * sqrt(dmax(c->Q + a * a * c->E * c->E, 0.0))) {
        c->L = 0.0;
        c->Q = s->vtheta * s->vtheta - cs * cs * a * a * c->E * c->E;
    }
}

/* Classical RK4 step of size h in Mino time (src/kerr.cpp:502-519). */
void orc_step_mino(double a, const orc_constants* c, orc_state* s, double h) {
    orc_derivs k[4];
    orc_state y = *s;
    static const double frac[4] = {0.0, 0.5, 0.5, 1.0};
    for (int i = 0; i < 4; ++i) {
        if (i > 0) {
            const double hh = frac[i] * h;
            y.r = s->r + hh * k[i - 1].dr;
            y.theta = s->theta + hh * k[i - 1].dtheta;
            y.phi = s->phi + hh * k[i - 1].dphi;
            y.vr = s->vr + hh * k[i - 1].dvr;
            y.vtheta = s->vtheta + hh * k[i - 1].dvtheta;
        }
        orc_derivatives(a, c, &y, &k[i]);
    }
    const double w = h / 6.0;
    s->t += w * (k[0].dt + 2.0 * k[1].dt + 2.0 * k[2].dt + k[3].dt);
    s->r += w * (k[0].dr + 2.0 * k[1].dr + 2.0 * k[2].dr + k[3].dr);
    s->theta += w * (k[0].dtheta + 2.0 * k[1].dtheta + 2.0 * k[2].dtheta + k[3].dtheta);
    s->phi += w * (k[0].dphi + 2.0 * k[1].dphi + 2.0 * k[2].dphi + k[3].dphi);
    s->vr += w * (k[0].dvr + 2.0 * k[1].dvr + 2.0 * k[2].dvr + k[3].dvr);
    s->vtheta += w * (k[0].dvtheta + 2.0 * k[1].dvtheta + 2.0 * k[2].dvtheta + k[3].dvtheta);
}

/* Re-project onto vr^2 = R, vtheta^2 = Theta outside a 5% turning zone (src/kerr.cpp:521-542). */
void orc_enforce_constraints(double a, const orc_constants* c, orc_state* s) {
    const double zone = 0.05;
    const double r = s->r;
    const double delta = r * r - 2.0 * r + a * a;
    const double P = c->E * (r * r + a * a) - a * c->L;
    const double x = c->L - a * c->E;
    const double K = c->mu * c->mu * r * r + x * x + c->Q;
    const double R = P * P - delta * K;
    if (R > zone * (P * P + fabs(delta) * K)) s->vr = copysign(sqrt(R), s->vr);
    const double sn = sin(s->theta), cs = cos(s->theta);
    const double cot2 = cs * cs / dmax(sn * sn, 1e-18);
    const double polar_mass = a * a * (c->mu * c->mu - c->E * c->E) * cs * cs;
    const double Th = c->Q - polar_mass - c->L * c->L * cot2;
    if (Th > zone * (fabs(c->Q) + fabs(polar_mass) + c->L * c->L * cot2)) s->vtheta = copysign(sqrt(Th), s->vtheta);
}

/* Heuristic Mino step bounding the relative change of r, sin(theta), phi and the
 * accelerations (src/kerr.cpp:563-575). */
double orc_photon_step_size(double a, const orc_constants* c, const orc_state* s, double tol) {
    orc_derivs d;
    orc_derivatives(a, c, s, &d);
    const double sn = fabs(sin(s->theta));
    const double cs = cos(s->theta);
    const double rs = is_naked(a) ? dmax(sqrt(s->r * s->r + a * a * cs * cs), 0.02) : s->r;
    const double t = tol * dclamp(rs / 8.0, 1.0, 4.0);
    double h = t / (fabs(d.dr) / rs + fabs(d.dtheta) / dmax(sn, 1e-4) + fabs(d.dphi) + 1e-6);
    h = dmin(h, sqrt(t * rs / (fabs(d.dvr) + 1e-6)));
    h = dmin(h, sqrt(t * dmax(sn, 1e-4) / (fabs(d.dvtheta) + 1e-6)));
    return h;
}

/* theta into [0, pi] by reflection through the pole (src/kerr.cpp:595-604). */
void orc_normalize_angles(orc_state* s) {
    s->theta = fmod(s->theta, 2.0 * ORC_PI);
    if (s->theta < 0.0) s->theta += 2.0 * ORC_PI;
    if (s->theta > ORC_PI) {
        s->theta = 2.0 * ORC_PI - s->theta;
        s->phi += ORC_PI;
        s->vtheta = -s->vtheta;
    }
}

/* Kerr-Schild Cartesian position and velocity (src/kerr.cpp:638-658). */
void orc_to_cartesian(double a, double r, double theta, double phi, double out[3]) {
    const double sn = sin(theta), cp = cos(phi), sp = sin(phi);
    out[0] = (r * cp - a * sp) * sn;
    out[1] = (r * sp + a * cp) * sn;
    out[2] = r * cos(theta);
}

void orc_cartesian_velocity(double a, double r, double theta, double phi, double dr, double dtheta,
                            double dphi, double out[3]) {
    const double sn = sin(theta), cs = cos(theta), cp = cos(phi), sp = sin(phi);
    const double re = dr * sn + r * cs * dtheta - a * sn * dphi;
    const double im = a * cs * dtheta + r * sn * dphi;
    out[0] = re * cp - im * sp;
    out[1] = re * sp + im * cp;
    out[2] = dr * cs - r * sn * dtheta;
}

/* -------------------------------------------------------- critical curve ---- */

/* Bardeen critical curve from spherical photon orbits, upper half then mirrored
 * (src/eht.cpp:52-80). Returns the point count written (<= cap). */
int orc_critical_curve(double a, double inclination, int samples, double* alpha, double* beta, int cap) {
    const double sinI = sin(inclination), cosI = cos(inclination);
    int n_out = 0;
    if (fabs(a) < 1e-6) {
        for (int k = 0; k < samples && n_out < cap; ++k, ++n_out) {
            const double psi = 2.0 * ORC_PI * k / samples;
            alpha[n_out] = sqrt(27.0) * cos(psi);
            beta[n_out] = sqrt(27.0) * sin(psi);
        }
        return n_out;
    }
    const double r1 = orc_photon_orbit_radius(a, 1), r2 = orc_photon_orbit_radius(a, 0);
    const int n = (samples > 16 ? samples : 16) * 8;
    int n_up = 0;
    double* ua = (double*)malloc(sizeof(double) * (size_t)(n + 1));
    double* ub = (double*)malloc(sizeof(double) * (size_t)(n + 1));
    for (int k = 0; k <= n; ++k) {
        const double x = 0.5 - 0.5 * cos(ORC_PI * k / n);
        const double r = r1 + (r2 - r1) * x;
        const double xi = (r * r * (3.0 - r) - a * a * (r + 1.0)) / (a * (r - 1.0));
        const double eta = r * r * r * (4.0 * a * a - r * (r - 3.0) * (r - 3.0)) / (a * a * (r - 1.0) * (r - 1.0));
        const double b2 = eta + a * a * cosI * cosI - xi * xi * cosI * cosI / (sinI * sinI);
        if (b2 < 0.0) continue;
        ua[n_up] = -xi / sinI;
        ub[n_up] = sqrt(b2);
        ++n_up;
    }
    for (int k = 0; k < n_up && n_out < cap; ++k, ++n_out) {
        alpha[n_out] = ua[k];
        beta[n_out] = ub[k];
    }
    for (int k = n_up - 1; k >= 0 && n_out < cap; --k, ++n_out) {
        alpha[n_out] = ua[k];
        beta[n_out] = -ub[k];
    }
    free(ua);
    free(ub);
    return n_out;
}

/* Distance from the centre to the curve along direction psi (src/eht.cpp:82-97). */
double orc_critical_radius(const double* alpha, const double* beta, int n, double psi) {
    const double dx = cos(psi), dy = sin(psi);
    double best = 0.0;
    for (int k = 0; k < n; ++k) {
        const int q = (k + 1) % n;
        const double ex = alpha[q] - alpha[k], ey = beta[q] - beta[k];
        const double det = ex * dy - ey * dx;
        if (fabs(det) < 1e-15) continue;
        const double t = (beta[k] * dx - alpha[k] * dy) / det;
        const double s = (ex * beta[k] - ey * alpha[k]) / det;
        if (t >= 0.0 && t <= 1.0 && s > 0.0) best = dmax(best, s);
    }
    return best;
}

/* The same spherical-orbit constants (xi, eta) = (L/E, Q/E^2), seen by a ZAMO pinhole at r_obs:
 * the photon's ZAMO-frame direction n has n_phi : n_theta : n_r = xi/varpi : sqrt(Theta)/sqrt(Sigma)
 * : sqrt(R)/sqrt(Sigma Delta), and the pinhole maps look = -n to (alpha, beta) = r_obs (n_phi,
 * -n_theta)/(-n_r) up to the sign conventions of orc_pinhole_launch. Tends to the Bardeen curve as
 * r_obs -> infinity. */
int orc_critical_curve_finite(double a, double r_obs, double theta_obs, int samples, double* alpha,
                              double* beta, int cap) {
    const double aa = fabs(a) < 1e-6 ? 1e-6 : a;
    const double r1 = orc_photon_orbit_radius(aa, 1), r2 = orc_photon_orbit_radius(aa, 0);
    const orc_metric m = metric_at(aa, r_obs, theta_obs);
    const double sn = sin(theta_obs), cs = cos(theta_obs);
    const double varpi = sqrt(m.A / m.sigma) * sn;
    const int n = (samples > 16 ? samples : 16) * 8;
    double* ua = (double*)malloc(sizeof(double) * (size_t)(n + 1));
    double* ub = (double*)malloc(sizeof(double) * (size_t)(n + 1));
    int n_up = 0, n_out = 0;
    for (int k = 0; k <= n; ++k) {
        const double x = 0.5 - 0.5 * cos(ORC_PI * k / n);
        const double r = r1 + (r2 - r1) * x;
        const double xi = (r * r * (3.0 - r) - aa * aa * (r + 1.0)) / (aa * (r - 1.0));
        const double eta = r * r * r * (4.0 * aa * aa - r * (r - 3.0) * (r - 3.0)) / (aa * aa * (r - 1.0) * (r - 1.0));
        orc_constants c = {1.0, xi, eta, 0.0};
        const double R = orc_radial_potential(aa, &c, r_obs);
        const double Th = orc_polar_potential(aa, &c, theta_obs);
        if (R <= 0.0 || Th < 0.0) continue;
        const double eloc = (1.0 - m.omega * xi);  /* common positive factor dropped below */
        const double nr = sqrt(R) / sqrt(m.sigma * m.delta) / eloc;
        const double nth = sqrt(Th) / sqrt(m.sigma) / eloc;
        const double nph = xi / varpi / eloc;
        /* look = -n; pinhole look ~ (-1, -beta/r, alpha/r) => alpha = r (-nph)/nr, |beta| = r nth/nr */
        ua[n_up] = r_obs * (-nph) / nr;
        ub[n_up] = r_obs * nth / nr;
        ++n_up;
    }
    (void)cs;
    for (int k = 0; k < n_up && n_out < cap; ++k, ++n_out) {
        alpha[n_out] = ua[k];
        beta[n_out] = ub[k];
    }
    for (int k = n_up - 1; k >= 0 && n_out < cap; --k, ++n_out) {
        alpha[n_out] = ua[k];
        beta[n_out] = -ub[k];
    }
    free(ua);
    free(ub);
    return n_out;
}

/* ------------------------------------------------------------ tracers ---- */

/* ZAMO pinhole: look = normalize(-1, -beta/r_obs, alpha/r_obs) on the frame's (r, theta, phi) axes,
 * launched through photonFromFrame (src/kerr.cpp:458-483). */
void orc_pinhole_launch(const orc_scene* sc, double alpha, double beta, orc_constants* c, orc_state* s) {
    double u[4];
    orc_frame f;
    orc_zamo_four_velocity(sc->a, sc->r_obs, sc->theta_obs, u);
    orc_observer_frame(sc->a, sc->r_obs, sc->theta_obs, u, &f);
    const double lr = -1.0, lt = -beta / sc->r_obs, lp = alpha / sc->r_obs;
    const double n = sqrt(lr * lr + lt * lt + lp * lp);
    const double look[3] = {lr / n, lt / n, lp / n};
    orc_photon_from_frame(sc->a, sc->r_obs, sc->theta_obs, sc->phi_obs, &f, look, c, s);
}

/* Thin-disk emission at the crossing radius rc: gas on prograde circular orbits,
 * g = sqrt(-(g_tt + 2 g_tphi W + g_phiphi W^2)) / (E - L W) (src/trajectory.cpp:311-318).
 * Returns 0 when the orbit is not timelike there. */
static int disk_redshift(double a, double E, double L, double rc, double* g) {
    const double w = orc_circular_omega(a, rc, 1);
    const double gtt = -(1.0 - 2.0 / rc), gtp = -2.0 * a / rc, gpp = rc * rc + a * a + 2.0 * a * a / rc;
    const double norm = -(gtt + 2.0 * gtp * w + gpp * w * w);
    if (!(norm > 0.0)) return 0;
    *g = sqrt(norm) / (E - L * w);
    return 1;
}

static double wrap_2pi(double x) {
    const double t = 2.0 * ORC_PI;
    double y = x - t * floor(x / t);
    if (y >= t) y -= t;
    return y;
}

/* Escape direction: the backward tangent -d(x)/d(tau), normalized, as (theta_inf, phi_inf)
 * (tests/test_kerr.cpp:276-280 direction, src/trajectory.cpp:383-392 sign). */
static void escape_direction(double a, const orc_constants* c, const orc_state* s, double* th, double* ph) {
    orc_derivs d;
    orc_derivatives(a, c, s, &d);
    double v[3];
    orc_cartesian_velocity(a, s->r, s->theta, s->phi, s->vr, s->vtheta, d.dphi, v);
    const double n = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    const double dx = -v[0] / n, dy = -v[1] / n, dz = -v[2] / n;
    *th = acos(dclamp(dz, -1.0, 1.0));
    *ph = atan2(dy, dx);
}

int orc_no_radial_root_below(double a, double E, double L, double Q, double r, double eps) {
    /* R(r) = E^2 r^4 + c2 r^2 + c1 r + c0 for a photon; expand about x0 = r_+(1 + eps) and bound
     * the cubic part from below on [x0, r]. */
    const double x0 = orc_horizon_radius(a) * (1.0 + eps);
    const double w = r - x0;
    if (w <= 0.0) return 1;
    const double xx = L - a * E, K = xx * xx + Q;
    const double c4 = E * E, c2 = -(2.0 * a * E * xx + K), c1 = 2.0 * K, c0 = -a * a * Q;
    const double R0 = ((c4 * x0 * x0 + c2) * x0 + c1) * x0 + c0;
    const double R1 = (4.0 * c4 * x0 * x0 + 2.0 * c2) * x0 + c1;
    const double R2 = 6.0 * c4 * x0 * x0 + c2;
    const double R3 = 4.0 * c4 * x0;
    const double lower = R0 - w * dmax(0.0, -R1) - w * w * dmax(0.0, -R2) - w * w * w * dmax(0.0, -R3);
    return lower > 0.0;
}

static void ray_init(orc_ray* out) {
    memset(out, 0, sizeof(*out));
    out->outcome = ORC_UNFINISHED;
    out->r_disk = out->phi_disk = out->g = out->theta_inf = out->phi_inf = NAN;
}

/* Sigma below which a ray has struck the ring singularity (shaders/trace.frag:1773-1778). */
#define ORC_RING_SIGMA 4e-4

static double effective_escape(const orc_scene* sc) { return dmax(sc->r_escape, 1.5 * sc->r_obs); }
static double disk_inner(const orc_scene* sc) {
    return sc->r_disk_in > 0.0 ? sc->r_disk_in : orc_isco_radius(sc->a, 1);
}

/* The reference loop shape (src/trajectory.cpp:259-392) at tolerance sc->tol, with the scene's
 * capture and escape radii. The escape point is interpolated linearly to r_escape. */
static void trace_rk4(const orc_scene* sc, orc_constants c, orc_state s, orc_ray* out) {
    out->E = c.E, out->L = c.L, out->Q = c.Q;
    const double a = sc->a;
    const int naked = is_naked(a);
    const double r_cap = orc_horizon_radius(a) * (1.0 + sc->capture_eps);
    const double r_esc = effective_escape(sc);
    const double r_in = disk_inner(sc), r_out = sc->r_disk_out;
    const double half_pi = 0.5 * ORC_PI;
    for (int i = 0; i < sc->max_steps; ++i) {
        const orc_state prev = s;
        orc_step_mino(a, &c, &s, -orc_photon_step_size(a, &c, &s, sc->tol));
        orc_normalize_angles(&s);
        orc_enforce_constraints(a, &c, &s);
        out->steps = i + 1;
        if (!isfinite(s.r)) return;
        if ((prev.theta - half_pi) * (s.theta - half_pi) < 0.0) {
            const double f = (prev.theta - half_pi) / (prev.theta - s.theta);
            const double rc = prev.r + f * (s.r - prev.r);
            double g;
            if (rc >= r_in && rc <= r_out && disk_redshift(a, c.E, c.L, rc, &g)) {
                out->outcome = ORC_DISK;
                out->r_disk = rc;
                out->phi_disk = wrap_2pi(prev.phi + f * (s.phi - prev.phi));
                out->g = g;
                return;
            }
        }
        if (naked) {
            const double cs = cos(s.theta);
            if (s.r * s.r + a * a * cs * cs < ORC_RING_SIGMA) {
                out->outcome = ORC_RING;
                return;
            }
        } else if (s.r < r_cap && s.r < prev.r) {
            out->outcome = ORC_CAPTURED;
            return;
        }
        const double r_far = naked ? -r_esc : -INFINITY;
        if ((s.r > r_esc && s.r > prev.r) || (s.r < r_far && s.r < prev.r)) {
            const double target = s.r > 0.0 ? r_esc : r_far;
            orc_state x = s;
            if (fabs(s.theta - prev.theta) < 1.0) {
                const double f = (target - prev.r) / (s.r - prev.r);
                x.r = target;
                x.theta = prev.theta + f * (s.theta - prev.theta);
                x.phi = prev.phi + f * (s.phi - prev.phi);
                x.vr = prev.vr + f * (s.vr - prev.vr);
                x.vtheta = prev.vtheta + f * (s.vtheta - prev.vtheta);
            }
            out->outcome = s.r > 0.0 ? ORC_ESCAPED : ORC_ESCAPED_BEYOND;
            escape_direction(a, &c, &x, &out->theta_inf, &out->phi_inf);
            return;
        }
    }
}

/* Dormand-Prince 5(4) tableau (Dormand & Prince 1980), its 4th-order continuous extension
 * (Shampine 1986, as in Hairer-Norsett-Wanner's DOPRI5), and error weights b - b*. */
static const double A21 = 1.0 / 5.0;
static const double A31 = 3.0 / 40.0, A32 = 9.0 / 40.0;
static const double A41 = 44.0 / 45.0, A42 = -56.0 / 15.0, A43 = 32.0 / 9.0;
static const double A51 = 19372.0 / 6561.0, A52 = -25360.0 / 2187.0, A53 = 64448.0 / 6561.0, A54 = -212.0 / 729.0;
static const double A61 = 9017.0 / 3168.0, A62 = -355.0 / 33.0, A63 = 46732.0 / 5247.0, A64 = 49.0 / 176.0,
                    A65 = -5103.0 / 18656.0;
static const double B1 = 35.0 / 384.0, B3 = 500.0 / 1113.0, B4 = 125.0 / 192.0, B5 = -2187.0 / 6784.0,
                    B6 = 11.0 / 84.0;
static const double E1 = 71.0 / 57600.0, E3 = -71.0 / 16695.0, E4 = 71.0 / 1920.0, E5 = -17253.0 / 339200.0,
                    E6 = 22.0 / 525.0, E7 = -1.0 / 40.0;
static const double D1 = -12715105075.0 / 11282082432.0, D3 = 87487479700.0 / 32700410799.0,
                    D4 = -10690763975.0 / 1880347072.0, D5 = 701980252875.0 / 199316789632.0,
                    D6 = -1453857185.0 / 822651844.0, D7 = 69997945.0 / 29380423.0;

typedef struct { double v[5]; } vec5;  /* r, theta, phi, vr, vtheta */

static void rhs5(double a, const orc_constants* c, const vec5* y, vec5* k) {
    orc_state s = {0.0, y->v[0], y->v[1], y->v[2], y->v[3], y->v[4]};
    orc_derivs d;
    orc_derivatives(a, c, &s, &d);
    k->v[0] = d.dr;
    k->v[1] = d.dtheta;
    k->v[2] = d.dphi;
    k->v[3] = d.dvr;
    k->v[4] = d.dvtheta;
}

/* Dense output of component i at fraction sg of the step. */
static double dense(const double* y0, const double* y1, const vec5 k[7], double h, int i, double sg) {
    const double yd = y1[i] - y0[i];
    const double b = h * k[0].v[i] - yd;
    const double c4 = yd - h * k[6].v[i] - b;
    const double c5 = h * (D1 * k[0].v[i] + D3 * k[2].v[i] + D4 * k[3].v[i] + D5 * k[4].v[i] + D6 * k[5].v[i] +
                           D7 * k[6].v[i]);
    const double s1 = 1.0 - sg;
    return y0[i] + sg * (yd + s1 * (b + sg * (c4 + s1 * c5)));
}

/* Bisection for the fraction where component i of the dense output equals target. */
static double locate(const double* y0, const double* y1, const vec5 k[7], double h, int i, double target) {
    double lo = 0.0, hi = 1.0;
    const double f0 = y0[i] - target;
    for (int it = 0; it < 60; ++it) {
        const double mid = 0.5 * (lo + hi);
        const double fm = dense(y0, y1, k, h, i, mid) - target;
        if ((fm < 0.0) == (f0 < 0.0)) lo = mid; else hi = mid;
    }
    return 0.5 * (lo + hi);
}

static void trace_dp5(const orc_scene* sc, orc_constants c, orc_state s, orc_ray* out) {
    out->E = c.E, out->L = c.L, out->Q = c.Q;
    const double a = sc->a;
    const double rp = orc_horizon_radius(a);
    const double r_cap = rp * (1.0 + sc->capture_eps);
    const double r_esc = effective_escape(sc);
    const double r_in = disk_inner(sc), r_out = sc->r_disk_out;
    const double zone = dmin(0.05, 0.5 * (r_in - rp));
    const int naked = is_naked(a);
    const double r_far = naked ? -r_esc : -INFINITY;
    const double rtol = sc->tol, atol = sc->tol;
    const double half_pi = 0.5 * ORC_PI;

    vec5 y = {{s.r, s.theta, s.phi, s.vr, s.vtheta}};
    vec5 k[7];
    rhs5(a, &c, &y, &k[0]);
    double h = -orc_photon_step_size(a, &c, &s, dclamp(pow(rtol, 0.2), 1e-3, 0.05));
    int accepted = 0, rejected = 0, last_rejected = 0;
    while (accepted < sc->max_steps && rejected < sc->max_steps) {
        vec5 t, y5;
        for (int i = 0; i < 5; ++i) t.v[i] = y.v[i] + h * (A21 * k[0].v[i]);
        rhs5(a, &c, &t, &k[1]);
        for (int i = 0; i < 5; ++i) t.v[i] = y.v[i] + h * (A31 * k[0].v[i] + A32 * k[1].v[i]);
        rhs5(a, &c, &t, &k[2]);
        for (int i = 0; i < 5; ++i) t.v[i] = y.v[i] + h * (A41 * k[0].v[i] + A42 * k[1].v[i] + A43 * k[2].v[i]);
        rhs5(a, &c, &t, &k[3]);
        for (int i = 0; i < 5; ++i)
            t.v[i] = y.v[i] + h * (A51 * k[0].v[i] + A52 * k[1].v[i] + A53 * k[2].v[i] + A54 * k[3].v[i]);
        rhs5(a, &c, &t, &k[4]);
        for (int i = 0; i < 5; ++i)
            t.v[i] = y.v[i] + h * (A61 * k[0].v[i] + A62 * k[1].v[i] + A63 * k[2].v[i] + A64 * k[3].v[i] +
                                   A65 * k[4].v[i]);
        rhs5(a, &c, &t, &k[5]);
        for (int i = 0; i < 5; ++i)
            y5.v[i] = y.v[i] + h * (B1 * k[0].v[i] + B3 * k[2].v[i] + B4 * k[3].v[i] + B5 * k[4].v[i] +
                                    B6 * k[5].v[i]);
        rhs5(a, &c, &y5, &k[6]);
        double acc = 0.0;
        for (int i = 0; i < 5; ++i) {
            const double e = h * (E1 * k[0].v[i] + E3 * k[2].v[i] + E4 * k[3].v[i] + E5 * k[4].v[i] +
                                  E6 * k[5].v[i] + E7 * k[6].v[i]);
            const double scale = atol + rtol * dmax(fabs(y.v[i]), fabs(y5.v[i]));
            acc += (e / scale) * (e / scale);
        }
        const double err = sqrt(acc / 5.0);
        if (!(err <= 1.0)) {
            ++rejected;
            last_rejected = 1;
            h *= isfinite(err) ? dmax(0.2, 0.9 * pow(err, -0.2)) : 0.2;
            continue;
        }
        ++accepted;
        out->steps = accepted;
        out->rejected = rejected;
        const vec5 prev = y;
        y = y5;
        if (!isfinite(y.v[0])) return;
        /* Disk: theta crosses pi/2 within the step. */
        if ((prev.v[1] - half_pi) * (y.v[1] - half_pi) < 0.0) {
            const double sg = locate(prev.v, y.v, k, h, 1, half_pi);
            const double rc = dense(prev.v, y.v, k, h, 0, sg);
            double g;
            if (rc >= r_in && rc <= r_out && disk_redshift(a, c.E, c.L, rc, &g)) {
                out->outcome = ORC_DISK;
                out->r_disk = rc;
                out->phi_disk = wrap_2pi(dense(prev.v, y.v, k, h, 2, sg));
                out->g = g;
                return;
            }
        }
        const int falling = y.v[0] < prev.v[0];
        if (naked) {
            const double cs = cos(y.v[1]);
            if (y.v[0] * y.v[0] + a * a * cs * cs < ORC_RING_SIGMA) {
                out->outcome = ORC_RING;
                return;
            }
        } else if (falling && (y.v[0] < r_cap || (y.v[0] < rp + zone &&
                                                  orc_no_radial_root_below(a, c.E, c.L, c.Q, y.v[0],
                                                                           sc->capture_eps)))) {
            out->outcome = ORC_CAPTURED;
            return;
        }
        if ((!falling && y.v[0] > r_esc) || (falling && y.v[0] < r_far)) {
            const double target = falling ? r_far : r_esc;
            const double sg = locate(prev.v, y.v, k, h, 0, target);
            orc_state x = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
            x.r = dense(prev.v, y.v, k, h, 0, sg);
            x.theta = dense(prev.v, y.v, k, h, 1, sg);
            x.phi = dense(prev.v, y.v, k, h, 2, sg);
            x.vr = dense(prev.v, y.v, k, h, 3, sg);
            x.vtheta = dense(prev.v, y.v, k, h, 4, sg);
            out->outcome = falling ? ORC_ESCAPED_BEYOND : ORC_ESCAPED;
            escape_direction(a, &c, &x, &out->theta_inf, &out->phi_inf);
            return;
        }
        /* Pole reflection and constraint re-projection, carrying the FSAL derivative along. */
        vec5 kn = k[6];
        orc_state st = {0.0, y.v[0], y.v[1], y.v[2], y.v[3], y.v[4]};
        const double phi_before = st.phi;
        orc_normalize_angles(&st);
        if (st.phi != phi_before) kn.v[4] = -kn.v[4];  /* reflected: Theta'(theta) is odd */
        orc_enforce_constraints(a, &c, &st);
        y.v[0] = st.r, y.v[1] = st.theta, y.v[2] = st.phi, y.v[3] = st.vr, y.v[4] = st.vtheta;
        kn.v[0] = y.v[3];
        kn.v[1] = y.v[4];
        k[0] = kn;
        double fac = err > 0.0 ? 0.9 * pow(err, -0.2) : 5.0;
        fac = dclamp(fac, 0.2, last_rejected ? 1.0 : 5.0);
        h *= fac;
        last_rejected = 0;
    }
}

static void trace_launched(const orc_scene* sc, const orc_constants* c, const orc_state* s, orc_ray* out) {
    if (sc->method == ORC_METHOD_DP5) trace_dp5(sc, *c, *s, out);
    else trace_rk4(sc, *c, *s, out);
}

void orc_trace_ray(const orc_scene* sc, double alpha, double beta, orc_ray* out) {
    ray_init(out);
    orc_constants c;
    orc_state s;
    orc_pinhole_launch(sc, alpha, beta, &c, &s);
    trace_launched(sc, &c, &s, out);
}

/* A camera with an arbitrary frame (moving, or inside the horizon), as trajectory::traceRay takes it
 * (src/trajectory.cpp:214-247): photonFromFrame at the scene's camera position; inside the horizon a
 * photon with 2 r_+ E - a L < 0 crossed into the hole from the far side of the eternal spacetime and
 * ends on the horizon at once (src/trajectory.cpp:236-244); otherwise it is traced backward (it rises
 * through the horizon first). */
void orc_trace_framed(const orc_scene* sc, const orc_frame* f, const double look[3], orc_ray* out) {
    ray_init(out);
    orc_constants c;
    orc_state s;
    orc_photon_from_frame(sc->a, sc->r_obs, sc->theta_obs, sc->phi_obs, f, look, &c, &s);
    const double rh = orc_horizon_radius(sc->a);
    if (sc->r_obs < rh && 2.0 * rh * c.E - sc->a * c.L < 0.0) {
        out->E = c.E, out->L = c.L, out->Q = c.Q;
        out->outcome = ORC_CAPTURED;
        return;
    }
    trace_launched(sc, &c, &s, out);
}

/* -------------------------------------------------- thread-pool drivers ---- */

typedef struct {
    const orc_scene* sc;
    int64_t n;
    int width, height;
    double alpha_lo, alpha_hi, beta_lo, beta_hi;
    const double *a, *r_obs, *theta_obs, *alpha, *beta;  /* per-ray mode when alpha != NULL */
    int32_t* outcome;
    double *r_disk, *phi_disk, *g, *theta_inf, *phi_inf;
    int32_t* steps;
    atomic_long next;
    long chunk;
} pool_job;

static void store(pool_job* j, int64_t k, const orc_ray* r) {
    if (j->outcome) j->outcome[k] = r->outcome;
    if (j->r_disk) j->r_disk[k] = r->r_disk;
    if (j->phi_disk) j->phi_disk[k] = r->phi_disk;
    if (j->g) j->g[k] = r->g;
    if (j->theta_inf) j->theta_inf[k] = r->theta_inf;
    if (j->phi_inf) j->phi_inf[k] = r->phi_inf;
    if (j->steps) j->steps[k] = r->steps;
}

static void* pool_worker(void* arg) {
    pool_job* j = (pool_job*)arg;
    for (;;) {
        const long first = atomic_fetch_add(&j->next, j->chunk);
        if (first >= j->n) break;
        const long last = first + j->chunk < j->n ? first + j->chunk : j->n;
        for (long k = first; k < last; ++k) {
            orc_ray ray;
            if (j->alpha) {
                orc_scene sc = *j->sc;
                sc.a = j->a[k];
                sc.r_obs = j->r_obs[k];
                sc.theta_obs = j->theta_obs[k];
                orc_trace_ray(&sc, j->alpha[k], j->beta[k], &ray);
            } else {
                const int row = (int)(k / j->width), col = (int)(k % j->width);
                const double px = (j->alpha_hi - j->alpha_lo) / j->width;
                const double py = (j->beta_hi - j->beta_lo) / j->height;
                orc_trace_ray(j->sc, j->alpha_lo + (col + 0.5) * px, j->beta_hi - (row + 0.5) * py, &ray);
            }
            store(j, k, &ray);
        }
    }
    return NULL;
}

static void run_pool(pool_job* j, int nthreads) {
    if (nthreads < 1) nthreads = 1;
    atomic_init(&j->next, 0);
    pthread_t* tid = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
    for (int t = 1; t < nthreads; ++t) pthread_create(&tid[t], NULL, pool_worker, j);
    pool_worker(j);
    for (int t = 1; t < nthreads; ++t) pthread_join(tid[t], NULL);
    free(tid);
}

void orc_trace_frame(const orc_scene* sc, int width, int height, double alpha_lo, double alpha_hi,
                     double beta_lo, double beta_hi, int nthreads, int32_t* outcome, double* r_disk,
                     double* phi_disk, double* g, double* theta_inf, double* phi_inf, int32_t* steps) {
    pool_job j;
    memset(&j, 0, sizeof(j));
    j.sc = sc;
    j.n = (int64_t)width * height;
    j.width = width, j.height = height;
    j.alpha_lo = alpha_lo, j.alpha_hi = alpha_hi, j.beta_lo = beta_lo, j.beta_hi = beta_hi;
    j.outcome = outcome, j.r_disk = r_disk, j.phi_disk = phi_disk, j.g = g;
    j.theta_inf = theta_inf, j.phi_inf = phi_inf, j.steps = steps;
    j.chunk = width;  /* one image row per grab, as the reference's row queue */
    run_pool(&j, nthreads);
}

void orc_trace_rays(const orc_scene* sc, int64_t n, const double* a, const double* r_obs,
                    const double* theta_obs, const double* alpha, const double* beta, int nthreads,
                    int32_t* outcome, double* r_disk, double* phi_disk, double* g, double* theta_inf,
                    double* phi_inf, int32_t* steps) {
    pool_job j;
    memset(&j, 0, sizeof(j));
    j.sc = sc;
    j.n = n;
    j.a = a, j.r_obs = r_obs, j.theta_obs = theta_obs, j.alpha = alpha, j.beta = beta;
    j.outcome = outcome, j.r_disk = r_disk, j.phi_disk = phi_disk, j.g = g;
    j.theta_inf = theta_inf, j.phi_inf = phi_inf, j.steps = steps;
    j.chunk = 16;
    run_pool(&j, nthreads);
}
