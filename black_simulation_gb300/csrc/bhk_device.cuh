// bhk_device.cuh -- device-side Kerr photon physics for sm_103a, templated on the arithmetic type.
//
// FP64 (double) functions restate the reference's kerr:: primitives operation for operation
// (src/kerr.cpp:157-658) so that the batched per-step mirrors and the FP64 tracer agree with the
// reference to rounding. The FP32 (float) specialisations of the right-hand side are the
// throughput path: own sine/cosine (Cody-Waite reduction + Taylor polynomials), one approximate
// reciprocal per evaluation, constants hoisted per ray.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace bhk {

constexpr double kPi = 3.14159265358979323846;
constexpr int kNoRay = -1;

// ----------------------------------------------------------------------------- scalar math ----

__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// sin r and cos r of the reduced argument of x (|x| below a few thousand), and the quadrant k (its
// low bits). Reduction x = k pi/2 + r with a two-constant
// Cody-Waite split of pi/2 (hi = pi/2 rounded to float, lo = the remainder), then polynomials on
// |r| <= pi/4: sin r = r + r^3 (s3 + s5 r^2 + s7 r^4), cos r = 1 + r^2 (c2 + c4 r^2 + c6 r^4 + c8 r^6),
// whose coefficients were fitted for this file to the least maximum relative error by Lawson's
// iteratively reweighted least squares (3.8e-9 for sin, 6.4e-11 for cos before FP32 rounding;
// 7.1e-8 relative and 6.5e-8 absolute after it, as the Taylor polynomials of one degree more).
// k is rounded by adding 1.5 * 2^23 (the integer lands in the low mantissa bits, which also give
// the quadrant): no float/int conversion instructions, which on this part issue to the narrow
// FP64 pipe.
__device__ __forceinline__ int sincos_reduced(float x, float* sr, float* cr) {
    const float shifted = fmaf(x, 0.636619772367581343f, 12582912.0f);
    const int q = __float_as_int(shifted);
    const float k = __fsub_rn(shifted, 12582912.0f);
    float r = fmaf(k, -1.57079637050628662109375f, x);
    r = fmaf(k, 4.37113900018624283e-8f, r);
    const float r2 = __fmul_rn(r, r);
    float ps = fmaf(r2, -1.9515282645509862e-4f, 8.332160757714382e-3f);     // s7, s5
    ps = fmaf(r2, ps, -1.6666654609479015e-1f);                               // s3
    *sr = fmaf(__fmul_rn(r, r2), ps, r);
    float pc = fmaf(r2, 2.4383566768620477e-5f, -1.3886681641998991e-3f);    // c8, c6
    pc = fmaf(r2, pc, 4.166662035693103e-2f);                                 // c4
    pc = fmaf(r2, pc, -4.9999999694474034e-1f);                               // c2
    *cr = fmaf(r2, pc, 1.0f);
    return q;
}

// sin x and cos x from the reduced pair: quadrant k mod 4 = 0, 1, 2, 3 gives
// (sin, cos) = (sr, cr), (cr, -sr), (-sr, -cr), (-cr, sr).
__device__ __forceinline__ void sincos_fast(float x, float* s, float* c) {
    float sr, cr;
    const int q = sincos_reduced(x, &sr, &cr);
    const float s0 = (q & 1) ? cr : sr;
    const float c0 = (q & 1) ? sr : cr;
    *s = (q & 2) ? -s0 : s0;
    *c = ((q + 1) & 2) ? -c0 : c0;
}

template <typename T>
struct Math;

template <>
struct Math<double> {
    static __device__ __forceinline__ void sc(double x, double* s, double* c) { sincos(x, s, c); }
    static __device__ __forceinline__ double div(double n, double d) { return n / d; }
};

template <>
struct Math<float> {
    static __device__ __forceinline__ void sc(float x, float* s, float* c) { sincos_fast(x, s, c); }
    static __device__ __forceinline__ float div(float n, float d) { return n * rcp_approx(d); }
};

// ------------------------------------------------------------------- FP64 kerr primitives ----

struct Cons { double E, L, Q, mu; };
struct St { double t, r, theta, phi, vr, vtheta; };
struct Der { double dt, dr, dtheta, dphi, dvr, dvtheta; };

__host__ __device__ __forceinline__ double dmaxd(double x, double y) { return x > y ? x : y; }
__host__ __device__ __forceinline__ double dmind(double x, double y) { return x < y ? x : y; }

__host__ __device__ __forceinline__ bool naked(double a) { return fabs(a) > 1.0; }

// r_+ (src/kerr.cpp:157-160).
__host__ __device__ __forceinline__ double horizon_radius(double a) {
    return naked(a) ? 0.0 : 1.0 + sqrt(dmaxd(0.0, 1.0 - a * a));
}

// Energy per unit mass of the circular equatorial orbit at r (Bardeen, Press & Teukolsky 1972), 1e30
// where there is none (src/kerr.cpp:122-129).
__host__ __device__ __forceinline__ double circular_energy(double a, double r, bool prograde) {
    const double sg = prograde ? 1.0 : -1.0, q = sqrt(r);
    const double den = r * q - 3.0 * q + 2.0 * sg * a;
    if (den <= 0.0) return 1e30;
    return (r * q - 2.0 * q + sg * a) / (pow(r, 0.75) * sqrt(den));
}

// The radius of least circular-orbit energy in [lo, hi]: the best of 4001 points of a geometric grid,
// then 80 golden-section steps between its neighbours (src/kerr.cpp:131-153). Out of line: on the
// device it runs once per frame (or per explicit ray past a = 1) and should not weigh on its callers'
// registers.
static __host__ __device__ __noinline__ double least_energy_radius(double a, bool prograde, double lo, double hi) {
    const int n = 4000;
    int best = 0;
    double best_e = 1e30;
    for (int k = 0; k <= n; ++k) {
        const double e = circular_energy(a, lo * pow(hi / lo, static_cast<double>(k) / n), prograde);
        if (e < best_e) {
            best_e = e;
            best = k;
        }
    }
    double x0 = lo * pow(hi / lo, (best > 1 ? best - 1 : 0) / static_cast<double>(n));
    double x1 = lo * pow(hi / lo, (best + 1 < n ? best + 1 : n) / static_cast<double>(n));
    const double gr = 0.5 * (sqrt(5.0) - 1.0);
    for (int k = 0; k < 80; ++k) {
        const double u = x1 - gr * (x1 - x0), v = x0 + gr * (x1 - x0);
        if (circular_energy(a, u, prograde) < circular_energy(a, v, prograde)) x1 = v;
        else x0 = u;
    }
    return 0.5 * (x0 + x1);
}

// Circular equatorial photon orbit (src/kerr.cpp:192-206): 2 (1 + cos(2/3 acos(-+a))); past a = 1 the
// retrograde root of r (r - 3)^2 = 4 a^2 by bisection, and no prograde one (0).
__host__ __device__ __forceinline__ double photon_orbit_radius(double a, bool prograde) {
    if (naked(a)) {
        if (prograde) return 0.0;
        double lo = 3.0, hi = 3.0 + 2.0 * fabs(a);
        for (int k = 0; k < 100; ++k) {
            const double m = 0.5 * (lo + hi);
            if (m * (m - 3.0) * (m - 3.0) < 4.0 * a * a) lo = m; else hi = m;
        }
        return 0.5 * (lo + hi);
    }
    return 2.0 * (1.0 + cos(2.0 / 3.0 * acos((prograde ? -1.0 : 1.0) * a)));
}

// Prograde/retrograde ISCO, Bardeen-Press-Teukolsky (src/kerr.cpp:179-190); past a = 1 the least
// energy of circular orbits, prograde over [1e-3, 30], retrograde from just outside the retrograde
// photon orbit to 60 (src/kerr.cpp:180-185).
__host__ __device__ __forceinline__ double isco_radius(double a, bool prograde) {
    if (naked(a))
        return prograde ? least_energy_radius(a, true, 1e-3, 30.0)
                        : least_energy_radius(a, false, photon_orbit_radius(a, false) * 1.0001, 60.0);
    const double z1 = 1.0 + cbrt(1.0 - a * a) * (cbrt(1.0 + a) + cbrt(1.0 - a));
    const double z2 = sqrt(3.0 * a * a + z1 * z1);
    const double w = sqrt(dmaxd(0.0, (3.0 - z1) * (3.0 + z1 + 2.0 * z2)));
    return prograde ? 3.0 + z2 - w : 3.0 + z2 + w;
}

// Keplerian angular velocity (src/kerr.cpp:296-299).
__device__ __forceinline__ double circular_omega(double a, double r, bool prograde) {
    const double s = prograde ? 1.0 : -1.0;
    return s / (r * sqrt(r) + s * a);
}

// Covariant Kerr-Schild metric (src/kerr.cpp:238-254).
__host__ __device__ __forceinline__ void metric_tensor(double a, double r, double theta, double g[4][4]) {
    double sn, cs;
    sincos(theta, &sn, &cs);
    const double sn2 = sn * sn;
    const double sigma = r * r + a * a * cs * cs;
    const double rra = r * r + a * a;
    const double A = rra * rra - a * a * (r * r - 2.0 * r + a * a) * sn2;
    const double f = 2.0 * r / sigma;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) g[i][j] = 0.0;
    g[0][0] = -(1.0 - f);
    g[0][1] = g[1][0] = f;
    g[0][3] = g[3][0] = -f * a * sn2;
    g[1][1] = 1.0 + f;
    g[1][3] = g[3][1] = -a * sn2 * (1.0 + f);
    g[2][2] = sigma;
    g[3][3] = A * sn2 / sigma;
}

__host__ __device__ __forceinline__ double metric_dot(const double g[4][4], const double* x, const double* y) {
    double acc = 0.0;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc += g[i][j] * x[i] * y[j];
    return acc;
}

struct MetricAt { double sigma, delta, A, omega; };

// (src/kerr.cpp:227-236)
__host__ __device__ __forceinline__ MetricAt metric_at(double a, double r, double theta) {
    double sn, cs;
    sincos(theta, &sn, &cs);
    MetricAt m;
    m.sigma = r * r + a * a * cs * cs;
    m.delta = r * r - 2.0 * r + a * a;
    const double rra = r * r + a * a;
    m.A = rra * rra - a * a * m.delta * sn * sn;
    m.omega = 2.0 * a * r / m.A;
    return m;
}

// (src/kerr.cpp:323-329)
__device__ __forceinline__ double inflow_factor(double P, double vr, double delta, double K) {
    if (P * vr < 0.0) return K / (P - vr);
    const double d = fabs(delta) > 1e-12 ? delta : copysign(1e-12, delta);
    return (P + vr) / d;
}

// kerr::derivatives (src/kerr.cpp:331-351), including dt and the rest mass mu.
__device__ __forceinline__ Der derivatives(double a, const Cons& c, const St& s) {
    const double r = s.r;
    double sn, cs;
    sincos(s.theta, &sn, &cs);
    const double sn2 = dmaxd(sn * sn, 1e-18);
    const double a2 = a * a, mu2 = c.mu * c.mu;
    const double delta = r * r - 2.0 * r + a2;
    const double rra = r * r + a2;
    const double P = c.E * rra - a * c.L;
    const double x = c.L - a * c.E;
    const double K = mu2 * r * r + x * x + c.Q;
    const double inflow = inflow_factor(P, s.vr, delta, K);
    const double m = dmaxd(fabs(sn), 1e-9);
    const double ssc = (sn < 0.0 ? -m : m) * m * m;
    Der d;
    d.dr = s.vr;
    d.dtheta = s.vtheta;
    d.dvr = 2.0 * c.E * r * P - (r - 1.0) * K - delta * mu2 * r;
    d.dvtheta = sn * cs * a2 * (mu2 - c.E * c.E) + c.L * c.L * cs / ssc;
    d.dphi = a * inflow - a * c.E + c.L / sn2;
    d.dt = rra * inflow - a * (a * c.E * sn * sn - c.L) - s.vr;
    return d;
}

// R(r), Theta(theta) (src/kerr.cpp:353-363).
__device__ __forceinline__ double radial_potential(double a, const Cons& c, double r) {
    const double delta = r * r - 2.0 * r + a * a;
    const double P = c.E * (r * r + a * a) - a * c.L;
    const double x = c.L - a * c.E;
    return P * P - delta * (c.mu * c.mu * r * r + x * x + c.Q);
}
__device__ __forceinline__ double polar_potential(double a, const Cons& c, double theta) {
    double sn, cs;
    sincos(theta, &sn, &cs);
    return c.Q - cs * cs * (a * a * (c.mu * c.mu - c.E * c.E) + c.L * c.L / dmaxd(sn * sn, 1e-18));
}

// RK4 step (src/kerr.cpp:502-519).
__device__ __forceinline__ void step_mino(double a, const Cons& c, St& s, double h) {
    const Der d1 = derivatives(a, c, s);
    St y = s;
    y.r = s.r + 0.5 * h * d1.dr; y.theta = s.theta + 0.5 * h * d1.dtheta; y.phi = s.phi + 0.5 * h * d1.dphi;
    y.vr = s.vr + 0.5 * h * d1.dvr; y.vtheta = s.vtheta + 0.5 * h * d1.dvtheta;
    const Der d2 = derivatives(a, c, y);
    y.r = s.r + 0.5 * h * d2.dr; y.theta = s.theta + 0.5 * h * d2.dtheta; y.phi = s.phi + 0.5 * h * d2.dphi;
    y.vr = s.vr + 0.5 * h * d2.dvr; y.vtheta = s.vtheta + 0.5 * h * d2.dvtheta;
    const Der d3 = derivatives(a, c, y);
    y.r = s.r + h * d3.dr; y.theta = s.theta + h * d3.dtheta; y.phi = s.phi + h * d3.dphi;
    y.vr = s.vr + h * d3.dvr; y.vtheta = s.vtheta + h * d3.dvtheta;
    const Der d4 = derivatives(a, c, y);
    const double w = h / 6.0;
    s.t += w * (d1.dt + 2.0 * d2.dt + 2.0 * d3.dt + d4.dt);
    s.r += w * (d1.dr + 2.0 * d2.dr + 2.0 * d3.dr + d4.dr);
    s.theta += w * (d1.dtheta + 2.0 * d2.dtheta + 2.0 * d3.dtheta + d4.dtheta);
    s.phi += w * (d1.dphi + 2.0 * d2.dphi + 2.0 * d3.dphi + d4.dphi);
    s.vr += w * (d1.dvr + 2.0 * d2.dvr + 2.0 * d3.dvr + d4.dvr);
    s.vtheta += w * (d1.dvtheta + 2.0 * d2.dvtheta + 2.0 * d3.dvtheta + d4.dvtheta);
}

// Null-constraint re-projection outside a 5% turning zone (src/kerr.cpp:521-542). Returns the
// state's new (vr, vtheta) through s.
__device__ __forceinline__ void enforce_constraints(double a, const Cons& c, St& s) {
    const double zone = 0.05;
    const double r = s.r;
    const double delta = r * r - 2.0 * r + a * a;
    const double P = c.E * (r * r + a * a) - a * c.L;
    const double x = c.L - a * c.E;
    const double K = c.mu * c.mu * r * r + x * x + c.Q;
    const double R = P * P - delta * K;
    if (R > zone * (P * P + fabs(delta) * K)) s.vr = copysign(sqrt(R), s.vr);
    double sn, cs;
    sincos(s.theta, &sn, &cs);
    const double cot2 = cs * cs / dmaxd(sn * sn, 1e-18);
    const double pm = a * a * (c.mu * c.mu - c.E * c.E) * cs * cs;
    const double Th = c.Q - pm - c.L * c.L * cot2;
    if (Th > zone * (fabs(c.Q) + fabs(pm) + c.L * c.L * cot2)) s.vtheta = copysign(sqrt(Th), s.vtheta);
}

// (src/kerr.cpp:563-575)
__device__ __forceinline__ double photon_step_size(double a, const Cons& c, const St& s, double tol) {
    const Der d = derivatives(a, c, s);
    double sn, cs;
    sincos(s.theta, &sn, &cs);
    sn = fabs(sn);
    const double rs = naked(a) ? dmaxd(sqrt(s.r * s.r + a * a * cs * cs), 0.02) : s.r;
    const double t = tol * fmin(fmax(rs / 8.0, 1.0), 4.0);
    double h = t / (fabs(d.dr) / rs + fabs(d.dtheta) / dmaxd(sn, 1e-4) + fabs(d.dphi) + 1e-6);
    h = dmind(h, sqrt(t * rs / (fabs(d.dvr) + 1e-6)));
    h = dmind(h, sqrt(t * dmaxd(sn, 1e-4) / (fabs(d.dvtheta) + 1e-6)));
    return h;
}

// Pole reflection (src/kerr.cpp:595-604). Returns true when it reflected.
__device__ __forceinline__ bool normalize_angles(St& s) {
    s.theta = fmod(s.theta, 2.0 * kPi);
    if (s.theta < 0.0) s.theta += 2.0 * kPi;
    if (s.theta > kPi) {
        s.theta = 2.0 * kPi - s.theta;
        s.phi += kPi;
        s.vtheta = -s.vtheta;
        return true;
    }
    return false;
}

// ZAMO 4-velocity (src/kerr.cpp:424-430).
__host__ __device__ __forceinline__ void zamo_four_velocity(double a, double r, double theta, double u[4]) {
    const MetricAt m = metric_at(a, r, theta);
    const double ut = sqrt(m.A / (m.sigma * m.delta));
    u[0] = ut; u[1] = 0.0; u[2] = 0.0; u[3] = m.omega * ut;
}

// Gram-Schmidt observer frame: slots filled in the order theta, phi, r (src/kerr.cpp:432-456).
__host__ __device__ __forceinline__ void observer_frame(double a, double r, double theta, const double u[4], double e[4][4]) {
    double g[4][4];
    metric_tensor(a, r, theta, g);
#pragma unroll
    for (int i = 0; i < 4; ++i) e[0][i] = u[i];
    const int coord[3] = {2, 3, 1};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        double w[4] = {0.0, 0.0, 0.0, 0.0};
        w[coord[k]] = 1.0;
        const double along = metric_dot(g, w, u);
#pragma unroll
        for (int i = 0; i < 4; ++i) w[i] += along * u[i];
#pragma unroll
        for (int j = 0; j < k; ++j) {
            const double p = metric_dot(g, w, e[coord[j]]);
#pragma unroll
            for (int i = 0; i < 4; ++i) w[i] -= p * e[coord[j]][i];
        }
        const double n = sqrt(dmaxd(metric_dot(g, w, w), 1e-300));
#pragma unroll
        for (int i = 0; i < 4; ++i) e[coord[k]][i] = w[i] / n;
    }
}

// photonFromFrame with the kAxisSnap rewrite (src/kerr.cpp:458-483, src/kerr.h:115).
__device__ __forceinline__ void photon_from_frame(double a, double r, double theta, double phi, const double e[4][4],
                                                  const double look[3], Cons& c, St& s) {
    double p[4], low[4], g[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i) p[i] = e[0][i] - look[0] * e[1][i] - look[1] * e[2][i] - look[2] * e[3][i];
    metric_tensor(a, r, theta, g);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        low[i] = 0.0;
#pragma unroll
        for (int j = 0; j < 4; ++j) low[i] += g[i][j] * p[j];
    }
    const double sigma = metric_at(a, r, theta).sigma;
    double sn, cs;
    sincos(theta, &sn, &cs);
    c.mu = 0.0;
    c.E = -low[0];
    c.L = low[3];
    s.t = 0.0; s.r = r; s.theta = theta; s.phi = phi;
    s.vr = sigma * p[1];
    s.vtheta = low[2];
    c.Q = s.vtheta * s.vtheta + cs * cs * (c.L * c.L / dmaxd(sn * sn, 1e-18) - a * a * c.E * c.E);
    if (fabs(c.L) < 3e-4 * sqrt(dmaxd(c.Q + a * a * c.E * c.E, 0.0))) {
        c.L = 0.0;
        c.Q = s.vtheta * s.vtheta - cs * cs * a * a * c.E * c.E;
    }
}

// launchFromZamo (src/kerr.cpp:365-407).
__device__ __forceinline__ void launch_from_zamo(double a, double r, double theta, double phi, const double v[3],
                                                 double mu, Cons& c, St& s) {
    const MetricAt m = metric_at(a, r, theta);
    double sn, cs;
    sincos(theta, &sn, &cs);
    double gamma = 1.0;
    if (mu > 0.0) {
        const double v2 = dmind(v[0] * v[0] + v[1] * v[1] + v[2] * v[2], 1.0 - 1e-12);
        gamma = 1.0 / sqrt(1.0 - v2);
    }
    c.mu = mu;
    c.L = gamma * v[2] * sqrt(m.A / m.sigma) * sn;
    c.E = gamma * sqrt(m.sigma * m.delta / m.A) + m.omega * c.L;
    s.t = 0.0; s.r = r; s.theta = theta; s.phi = phi;
    s.vr = gamma * v[0] * sqrt(m.sigma * m.delta);
    s.vtheta = gamma * v[1] * sqrt(m.sigma);
    if (mu == 0.0) {
        const double inv = 1.0 / c.E;
        c.E = 1.0;
        c.L *= inv;
        s.vr *= inv;
        s.vtheta *= inv;
    }
    c.Q = s.vtheta * s.vtheta + cs * cs * (a * a * (mu * mu - c.E * c.E) + c.L * c.L / dmaxd(sn * sn, 1e-18));
    if (mu == 0.0 && fabs(c.L) < 3e-4 * sqrt(dmaxd(c.Q + a * a, 0.0))) {
        c.L = 0.0;
        c.Q = s.vtheta * s.vtheta - cs * cs * a * a;
    }
}

// (src/kerr.cpp:651-658)
template <typename T>
__device__ __forceinline__ void cartesian_velocity(T a, T r, T theta, T phi, T dr, T dtheta, T dphi, T out[3]) {
    T sn, cs, sp, cp;
    Math<T>::sc(theta, &sn, &cs);
    Math<T>::sc(phi, &sp, &cp);
    const T re = dr * sn + r * cs * dtheta - a * sn * dphi;
    const T im = a * cs * dtheta + r * sn * dphi;
    out[0] = re * cp - im * sp;
    out[1] = re * sp + im * cp;
    out[2] = dr * cs - r * sn * dtheta;
}

// Thin disk of prograde circular orbits: g at crossing radius rc (src/trajectory.cpp:311-318).
__device__ __forceinline__ bool disk_redshift(double a, double E, double L, double rc, double* g) {
    const double w = circular_omega(a, rc, true);
    const double gtt = -(1.0 - 2.0 / rc), gtp = -2.0 * a / rc, gpp = rc * rc + a * a + 2.0 * a * a / rc;
    const double norm = -(gtt + 2.0 * gtp * w + gpp * w * w);
    if (!(norm > 0.0)) return false;
    *g = sqrt(norm) / (E - L * w);
    return true;
}

// True when R(r') > 0 on [r_+(1 + eps), r]: a photon falling there (backward in time) cannot turn
// back and reaches r_+(1 + eps). R = E^2 r^4 + c2 r^2 + c1 r + c0 is expanded about the capture
// radius and its cubic part bounded from below on the interval.
__device__ __forceinline__ bool no_radial_root_below(double a, double E, double L, double Q, double r, double eps) {
    const double x0 = horizon_radius(a) * (1.0 + eps);
    const double w = r - x0;
    if (w <= 0.0) return true;
    const double xx = L - a * E, K = xx * xx + Q;
    const double c4 = E * E, c2 = -(2.0 * a * E * xx + K), c1 = 2.0 * K, c0 = -a * a * Q;
    const double R0 = ((c4 * x0 * x0 + c2) * x0 + c1) * x0 + c0;
    const double R1 = (4.0 * c4 * x0 * x0 + 2.0 * c2) * x0 + c1;
    const double R2 = 6.0 * c4 * x0 * x0 + c2;
    const double R3 = 4.0 * c4 * x0;
    const double lower = R0 - w * dmaxd(0.0, -R1) - w * w * dmaxd(0.0, -R2) - w * w * w * dmaxd(0.0, -R3);
    return lower > 0.0;
}

// ------------------------------------------------------------- Dormand-Prince 5(4) tableau ----
// Dormand & Prince (1980); continuous extension of Shampine (1986) as in Hairer-Norsett-Wanner.

struct DP {
    static constexpr double a21 = 1.0 / 5.0;
    static constexpr double a31 = 3.0 / 40.0, a32 = 9.0 / 40.0;
    static constexpr double a41 = 44.0 / 45.0, a42 = -56.0 / 15.0, a43 = 32.0 / 9.0;
    static constexpr double a51 = 19372.0 / 6561.0, a52 = -25360.0 / 2187.0, a53 = 64448.0 / 6561.0,
                            a54 = -212.0 / 729.0;
    static constexpr double a61 = 9017.0 / 3168.0, a62 = -355.0 / 33.0, a63 = 46732.0 / 5247.0, a64 = 49.0 / 176.0,
                            a65 = -5103.0 / 18656.0;
    static constexpr double b1 = 35.0 / 384.0, b3 = 500.0 / 1113.0, b4 = 125.0 / 192.0, b5 = -2187.0 / 6784.0,
                            b6 = 11.0 / 84.0;
    static constexpr double e1 = 71.0 / 57600.0, e3 = -71.0 / 16695.0, e4 = 71.0 / 1920.0,
                            e5 = -17253.0 / 339200.0, e6 = 22.0 / 525.0, e7 = -1.0 / 40.0;
    static constexpr double d1 = -12715105075.0 / 11282082432.0, d3 = 87487479700.0 / 32700410799.0,
                            d4 = -10690763975.0 / 1880347072.0, d5 = 701980252875.0 / 199316789632.0,
                            d6 = -1453857185.0 / 822651844.0, d7 = 69997945.0 / 29380423.0;
};

// Per-ray constants of the photon right-hand side, hoisted out of the step (mu = 0).
template <typename T>
struct RayC {
    T a, a2, E, aE, aL, L, K, twoE, L2, nA2E2, Q;
    __device__ __forceinline__ void set(double a_, double E_, double L_, double Q_) {
        const double x = L_ - a_ * E_;
        a = T(a_); a2 = T(a_ * a_); E = T(E_); aE = T(a_ * E_); aL = T(a_ * L_); L = T(L_);
        K = T(x * x + Q_); twoE = T(2.0 * E_); L2 = T(L_ * L_); nA2E2 = T(-(a_ * a_) * E_ * E_); Q = T(Q_);
    }
    // From operands already rounded to T (K = (L - aE)^2 + Q formed in FP64 at launch).
    __device__ __forceinline__ void set_t(T a_, T E_, T L_, T Q_, T K_) {
        a = a_; a2 = a_ * a_; E = E_; aE = a_ * E_; aL = a_ * L_; L = L_; K = K_; twoE = T(2) * E_;
        L2 = L_ * L_; nA2E2 = -(a_ * a_) * (E_ * E_); Q = Q_;
    }
};

// The potentials R(r), Theta(theta) at an evaluated point and the 5% turning-zone thresholds of
// kerr::enforceConstraints (src/kerr.cpp:521-542), produced alongside a right-hand side.
template <typename T>
struct Proj {
    T R, Rz, Th, Thz;
};

// Right-hand side of the 5-component Mino system y = (r, theta, phi, vr, vtheta), photon (mu = 0):
// kerr::derivatives restated (src/kerr.cpp:331-351). With kProj it also returns the potentials for
// the null-constraint re-projection, sharing sin, cos, P and Delta; with dt (FP64) also dt/dlambda,
// the Kerr-Schild time, which the step carries as a passive extra component.
template <typename T, bool kProj = false>
__device__ __forceinline__ void rhs(const RayC<T>& c, const T y[5], T k[5], Proj<T>* pj = nullptr, T* dt = nullptr) {
    if constexpr (sizeof(T) == 4) {
        // The FP32 form, arranged for fused multiply-adds (the same terms, regrouped):
        //   Delta = (r^2 + a^2) - 2 r,  R'/2 = r (2 E P - K) + K,
        //   dphi = a inflow - a E + L / sin^2,  Theta'/2 = sin cos (-a^2 E^2 + (L / sin^2)^2).
        // theta enters only through sin^2, cos^2 and sin cos, so the quadrant's signs reduce to one:
        // with the reduced pair (sr, cr), sin^2 = (odd ? cr : sr)^2 and sin cos = (odd ? -1 : 1) sr cr.
        // Delta is not clamped away from 0: the FP32 tracer stays outside the capture zone, and a zero
        // there turns the state non-finite, which hands the ray to the FP64 continuation.
        // Every operation is spelled out (fmaf or a rounded intrinsic) so that no compilation of this
        // function contracts differently: the frame path and the launch kernel must agree bit for bit.
        const float r = y[0];
        float sr, cr;
        const bool odd = (sincos_reduced(y[1], &sr, &cr) & 1) != 0;
        const float m = odd ? cr : sr;                          // +-sin
        const float sc = __fmul_rn(odd ? -sr : sr, cr);         // sin cos
        // No clamp on sin^2: it is 0 only with theta exactly on a pole, where L / sin^2 is not finite
        // (0 * inf for the L = 0 rays that cross the axis; rays with L != 0 turn before the pole), so
        // such a stage makes the step's error non-finite and the step is rejected and retried shorter.
        const float inv2 = rcp_approx(__fmul_rn(m, m));
        const float li2 = __fmul_rn(c.L, inv2);                 // L / sin^2
        const float rra = fmaf(r, r, c.a2);
        const float delta = fmaf(-2.0f, r, rra);
        const float P = fmaf(c.E, rra, -c.aL);
        const bool opposite = __fmul_rn(P, y[3]) < 0.0f;
        const float num = opposite ? c.K : __fadd_rn(P, y[3]);
        const float den = opposite ? __fsub_rn(P, y[3]) : delta;
        const float inflow = __fmul_rn(num, rcp_approx(den));
        k[0] = y[3];
        k[1] = y[4];
        k[2] = fmaf(c.a, inflow, fmaf(c.L, inv2, -c.aE));
        k[3] = fmaf(r, fmaf(c.twoE, P, -c.K), c.K);
        k[4] = __fmul_rn(sc, fmaf(li2, li2, c.nA2E2));
        if constexpr (kProj) {
            const float P2 = __fmul_rn(P, P);
            pj->R = fmaf(-delta, c.K, P2);
            pj->Rz = __fmul_rn(0.05f, fmaf(fabsf(delta), c.K, P2));
            const float cm = odd ? sr : cr;                     // +-cos
            const float cs2 = __fmul_rn(cm, cm);
            const float l2cot2 = __fmul_rn(cs2, __fmul_rn(c.L, li2));  // L^2 cot^2
            const float pm = __fmul_rn(c.nA2E2, cs2);
            pj->Th = __fsub_rn(fmaf(-c.nA2E2, cs2, c.Q), l2cot2);
            pj->Thz = __fmul_rn(0.05f, __fadd_rn(__fadd_rn(fabsf(c.Q), fabsf(pm)), l2cot2));
        }
        (void)dt;
    } else {
        const T r = y[0];
        T sn, cs;
        Math<T>::sc(y[1], &sn, &cs);
        const T delta = r * r - T(2) * r + c.a2;
        const T rra = r * r + c.a2;
        const T P = c.E * rra - c.aL;
        const bool opposite = P * y[3] < T(0);
        const T dcl = fabs(delta) > T(1e-12) ? delta : copysign(T(1e-12), delta);
        const T num = opposite ? c.K : P + y[3];
        const T den = opposite ? P - y[3] : dcl;
        const T inflow = Math<T>::div(num, den);
        const T m = fmax(fabs(sn), T(1e-9));
        k[0] = y[3];
        k[1] = y[4];
        k[3] = c.twoE * r * P - (r - T(1)) * c.K;
        const T ssc = (sn < T(0) ? -m : m) * m * m;
        const T sn2 = fmax(sn * sn, T(1e-18));
        const T inv2 = T(1) / sn2;
        k[4] = sn * cs * c.nA2E2 + c.L2 * cs / ssc;
        k[2] = c.a * inflow - c.aE + c.L / sn2;
        if (dt) *dt = rra * inflow - c.a * (c.aE * sn * sn - c.L) - y[3];
        if constexpr (kProj) {
            const T P2 = P * P;
            pj->R = P2 - delta * c.K;
            pj->Rz = T(0.05) * (P2 + fabs(delta) * c.K);
            const T cs2 = cs * cs;
            const T cot2 = cs2 * inv2;
            const T pm = c.nA2E2 * cs2;
            pj->Th = c.Q - pm - c.L2 * cot2;
            pj->Thz = T(0.05) * (fabs(c.Q) + fabs(pm) + c.L2 * cot2);
        }
    }
}

__device__ __forceinline__ float sqrt_approx(float x) {
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Dense output of a passive component (its stage derivatives kt[0..6]) at fraction sg of a step.
__device__ __forceinline__ double dense1(double y0, double y1, const double kt[7], double h, double sg) {
    const double yd = y1 - y0;
    const double b = h * kt[0] - yd;
    const double c4 = yd - h * kt[6] - b;
    const double c5 = h * (DP::d1 * kt[0] + DP::d3 * kt[2] + DP::d4 * kt[3] + DP::d5 * kt[4] + DP::d6 * kt[5] +
                           DP::d7 * kt[6]);
    const double s1 = 1.0 - sg;
    return y0 + sg * (yd + s1 * (b + sg * (c4 + s1 * c5)));
}

// Dense output of one component at fraction sg of a step (continuous extension above).
template <typename T>
__device__ __forceinline__ T dense(T y0, T y1, const T k[7][5], T h, int i, T sg) {
    const T yd = y1 - y0;
    const T b = h * k[0][i] - yd;
    const T c4 = yd - h * k[6][i] - b;
    const T c5 = h * (T(DP::d1) * k[0][i] + T(DP::d3) * k[2][i] + T(DP::d4) * k[3][i] + T(DP::d5) * k[4][i] +
                      T(DP::d6) * k[5][i] + T(DP::d7) * k[6][i]);
    const T s1 = T(1) - sg;
    return y0 + sg * (yd + s1 * (b + sg * (c4 + s1 * c5)));
}

// One point of the analytic critical curve seen by a ZAMO pinhole at (r_obs, theta): the spherical
// photon orbit at x in [0, 1] along [r_pro, r_retro] (cosine spacing), its (xi, eta) of
// src/eht.cpp:52-80 launched back through the camera's frame. Returns false where that orbit's
// photons cannot reach the camera (R(r_obs) <= 0 or Theta(theta) < 0); beta >= 0 (upper half).
__device__ __forceinline__ bool critical_point(double a, double r_obs, double th, double x, double* alpha,
                                               double* beta) {
    const double aa = fabs(a) < 1e-6 ? 1e-6 : a;
    const double r1 = 2.0 * (1.0 + cos(2.0 / 3.0 * acos(-aa))), r2 = 2.0 * (1.0 + cos(2.0 / 3.0 * acos(aa)));
    const double r = r1 + (r2 - r1) * (0.5 - 0.5 * cos(kPi * x));
    const double xi = (r * r * (3.0 - r) - aa * aa * (r + 1.0)) / (aa * (r - 1.0));
    const double eta = r * r * r * (4.0 * aa * aa - r * (r - 3.0) * (r - 3.0)) / (aa * aa * (r - 1.0) * (r - 1.0));
    const Cons c{1.0, xi, eta, 0.0};
    const double R = radial_potential(aa, c, r_obs), Th = polar_potential(aa, c, th);
    const MetricAt m = metric_at(aa, r_obs, th);
    const double varpi = sqrt(m.A / m.sigma) * sin(th);
    const double eloc = 1.0 - m.omega * xi;
    const double nr = sqrt(fmax(R, 0.0)) / sqrt(m.sigma * m.delta) / eloc;
    const double nth = sqrt(fmax(Th, 0.0)) / sqrt(m.sigma) / eloc;
    const double nph = xi / varpi / eloc;
    *alpha = r_obs * (-nph) / nr;
    *beta = r_obs * nth / nr;
    return R > 0.0 && Th >= 0.0;
}

}  // namespace bhk
