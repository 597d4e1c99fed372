// bhk_steps.cu -- batched FP64 mirrors of the kerr:: per-step functions, one thread per item.
//
// Compiled with --fmad=false so each result differs from the reference's C++ (src/kerr.cpp)
// only by the last-bit differences of the device sin/cos/sqrt/cbrt.
#include "bhk_device.cuh"
#include "bhk_internal.h"

namespace bhk {

namespace {

constexpr int kBlock = 128;

__device__ __forceinline__ Cons ld(const bhk_constants& c) { return {c.E, c.L, c.Q, c.mu}; }
__device__ __forceinline__ St ld(const bhk_state& s) { return {s.t, s.r, s.theta, s.phi, s.vr, s.vtheta}; }
__device__ __forceinline__ void st(const St& s, bhk_state& o) {
    o.t = s.t; o.r = s.r; o.theta = s.theta; o.phi = s.phi; o.vr = s.vr; o.vtheta = s.vtheta;
}
__device__ __forceinline__ void st(const Cons& c, bhk_constants& o) { o.E = c.E; o.L = c.L; o.Q = c.Q; o.mu = c.mu; }

#define BHK_FOR(n) for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < (n); \
                        i += static_cast<int64_t>(gridDim.x) * blockDim.x)

__global__ void k_derivatives(double a, const bhk_constants* c, const bhk_state* s, bhk_derivatives_t* d, int64_t n) {
    BHK_FOR(n) {
        const Der r = derivatives(a, ld(c[i]), ld(s[i]));
        d[i].dt = r.dt; d[i].dr = r.dr; d[i].dtheta = r.dtheta;
        d[i].dphi = r.dphi; d[i].dvr = r.dvr; d[i].dvtheta = r.dvtheta;
    }
}

__global__ void k_step_mino(double a, const bhk_constants* c, bhk_state* s, const double* h, int64_t n) {
    BHK_FOR(n) {
        St x = ld(s[i]);
        step_mino(a, ld(c[i]), x, h[i]);
        st(x, s[i]);
    }
}

__global__ void k_step_size(double a, const bhk_constants* c, const bhk_state* s, double tol, double* h, int64_t n) {
    BHK_FOR(n) h[i] = photon_step_size(a, ld(c[i]), ld(s[i]), tol);
}

__global__ void k_enforce(double a, const bhk_constants* c, bhk_state* s, int64_t n) {
    BHK_FOR(n) {
        St x = ld(s[i]);
        enforce_constraints(a, ld(c[i]), x);
        st(x, s[i]);
    }
}

__global__ void k_normalize(bhk_state* s, int64_t n) {
    BHK_FOR(n) {
        St x = ld(s[i]);
        normalize_angles(x);
        st(x, s[i]);
    }
}

__global__ void k_potentials(double a, const bhk_constants* c, const bhk_state* s, double* R, double* Th, int64_t n) {
    BHK_FOR(n) {
        const Cons cc = ld(c[i]);
        if (R) R[i] = radial_potential(a, cc, s[i].r);
        if (Th) Th[i] = polar_potential(a, cc, s[i].theta);
    }
}

__global__ void k_frame(double a, const double* r, const double* th, const double* u, bhk_frame* f, int64_t n) {
    BHK_FOR(n) {
        double uu[4], e[4][4];
        if (u) {
            for (int k = 0; k < 4; ++k) uu[k] = u[4 * i + k];
        } else {
            zamo_four_velocity(a, r[i], th[i], uu);
        }
        observer_frame(a, r[i], th[i], uu, e);
        for (int k = 0; k < 4; ++k)
            for (int j = 0; j < 4; ++j) f[i].e[k][j] = e[k][j];
    }
}

__global__ void k_photon(double a, double r, double th, double ph, const bhk_frame* f, const double* look,
                         bhk_constants* c, bhk_state* s, int64_t n) {
    __shared__ double e[4][4];
    if (threadIdx.x < 16) e[threadIdx.x / 4][threadIdx.x % 4] = f->e[threadIdx.x / 4][threadIdx.x % 4];
    __syncthreads();
    BHK_FOR(n) {
        const double lk[3] = {look[3 * i], look[3 * i + 1], look[3 * i + 2]};
        Cons cc;
        St ss;
        photon_from_frame(a, r, th, ph, e, lk, cc, ss);
        st(cc, c[i]);
        st(ss, s[i]);
    }
}

__global__ void k_zamo(double a, double r, double th, double ph, const double* v, double mu, bhk_constants* c,
                       bhk_state* s, int64_t n) {
    BHK_FOR(n) {
        const double vv[3] = {v[3 * i], v[3 * i + 1], v[3 * i + 2]};
        Cons cc;
        St ss;
        launch_from_zamo(a, r, th, ph, vv, mu, cc, ss);
        st(cc, c[i]);
        st(ss, s[i]);
    }
}

__global__ void k_cartesian(double a, const bhk_constants* c, const bhk_state* s, double* out, int64_t n) {
    BHK_FOR(n) {
        const St x = ld(s[i]);
        const Der d = derivatives(a, ld(c[i]), x);
        double v[3];
        cartesian_velocity<double>(a, x.r, x.theta, x.phi, x.vr, x.vtheta, d.dphi, v);
        out[3 * i] = v[0]; out[3 * i + 1] = v[1]; out[3 * i + 2] = v[2];
    }
}

int grid_for(int64_t n) {
    const int64_t g = (n + kBlock - 1) / kBlock;
    return static_cast<int>(g < 1 ? 1 : (g > 65535 * 8 ? 65535 * 8 : g));
}

// ---- trajectory::predict (src/trajectory.cpp:130-185): a massive particle's path in coordinate time ----

// kerr::stepCoordinateTime (src/kerr.cpp:544-560): RK4 on the Mino system divided by dt/dtau.
__device__ __forceinline__ void step_coordinate_time(double a, const Cons& c, St& s, double h) {
    auto f = [&](const St& x, double k[5]) {
        const Der d = derivatives(a, c, x);
        const double inv = 1.0 / d.dt;
        k[0] = d.dr * inv; k[1] = d.dtheta * inv; k[2] = d.dphi * inv; k[3] = d.dvr * inv; k[4] = d.dvtheta * inv;
    };
    auto off = [&](const double k[5], double w) {
        St o = s;
        o.r += w * k[0]; o.theta += w * k[1]; o.phi += w * k[2]; o.vr += w * k[3]; o.vtheta += w * k[4];
        return o;
    };
    double k1[5], k2[5], k3[5], k4[5];
    f(s, k1);
    f(off(k1, 0.5 * h), k2);
    f(off(k2, 0.5 * h), k3);
    f(off(k3, h), k4);
    s.t += h;
    s.r += h / 6.0 * (k1[0] + 2.0 * k2[0] + 2.0 * k3[0] + k4[0]);
    s.theta += h / 6.0 * (k1[1] + 2.0 * k2[1] + 2.0 * k3[1] + k4[1]);
    s.phi += h / 6.0 * (k1[2] + 2.0 * k2[2] + 2.0 * k3[2] + k4[2]);
    s.vr += h / 6.0 * (k1[3] + 2.0 * k2[3] + 2.0 * k3[3] + k4[3]);
    s.vtheta += h / 6.0 * (k1[4] + 2.0 * k2[4] + 2.0 * k3[4] + k4[4]);
}

// kerr::suggestedTimeStep (src/kerr.cpp:577-592): velocity and acceleration limits and a fraction of
// the local orbital period.
__device__ __forceinline__ double suggested_time_step(double a, const Cons& c, const St& s, double tol) {
    const Der d = derivatives(a, c, s);
    const double inv = 1.0 / d.dt;
    const double sn = dmaxd(fabs(sin(s.theta)), 1e-3);
    const double rate = fabs(d.dr * inv) / s.r + fabs(d.dtheta * inv) / sn + fabs(d.dphi * inv);
    double h = tol / dmaxd(rate, 1e-12);
    const double acc = fabs(d.dvr) * inv * inv / s.r + fabs(d.dvtheta) * inv * inv / sn;
    h = dmind(h, sqrt(tol / dmaxd(acc, 1e-30)));
    return dmind(h, 0.05 * 2.0 * kPi * s.r * sqrt(s.r));
}

__device__ __forceinline__ void ks_cartesian(double a, const St& s, double p[3]) {
    double st_, ct, sp, cp;
    sincos(s.theta, &st_, &ct);
    sincos(s.phi, &sp, &cp);
    p[0] = (s.r * cp - a * sp) * st_;
    p[1] = (s.r * sp + a * cp) * st_;
    p[2] = s.r * ct;
}

__device__ __forceinline__ double angle_between(const double x[3], const double y[3]) {
    const double lx = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]), ly = sqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
    const double c = (x[0] * y[0] + x[1] * y[1] + x[2] * y[2]) / dmaxd(lx * ly, 1e-300);
    return acos(dmind(dmaxd(c, -1.0), 1.0));
}

__global__ void k_predict(double a, const bhk_constants* cin, const bhk_state* sin_, int64_t n, double max_time,
                          double min_spacing, int32_t max_points, double surface, double escape_radius,
                          bhk_state* s_out, bhk_path_out out) {
    BHK_FOR(n) {
        const Cons c = ld(cin[i]);
        St s = ld(sin_[i]);
        const double rh = surface > 0.0 ? surface - 0.02 : horizon_radius(a);
        const double t0 = s.t;
        double rmin = s.r, rmax = s.r;
        double last[3], prev_pos[3], p[3];
        ks_cartesian(a, s, last);
        double* pts = out.points ? out.points + 3 * static_cast<int64_t>(max_points + 1) * i : nullptr;
        if (pts) {  // the start is always the path's first point
            pts[0] = last[0]; pts[1] = last[1]; pts[2] = last[2];
        }
        int count = 1;
        prev_pos[0] = last[0]; prev_pos[1] = last[1]; prev_pos[2] = last[2];
        double swept = 0.0, first_sweep = -1.0, prev_vr = s.vr;
        int periapses = 0, fate = BHK_FATE_BOUND;
        for (int guard = 0; guard < 400000 && s.t - t0 < max_time; ++guard) {
            const double h = dmind(suggested_time_step(a, c, s, 0.01), max_time - (s.t - t0));
            step_coordinate_time(a, c, s, h);
            normalize_angles(s);
            if (!isfinite(s.r) || s.r < rh + 0.02) {
                fate = surface > 0.0 ? BHK_FATE_HITS_SURFACE : BHK_FATE_PLUNGES;
                break;
            }
            if (s.r > escape_radius) {
                fate = BHK_FATE_ESCAPES;
                break;
            }
            rmin = dmind(rmin, s.r);
            rmax = dmaxd(rmax, s.r);
            ks_cartesian(a, s, p);
            swept += angle_between(prev_pos, p);
            prev_pos[0] = p[0]; prev_pos[1] = p[1]; prev_pos[2] = p[2];
            if (prev_vr < 0.0 && s.vr >= 0.0) {  // periapsis: the radial velocity turns outward
                if (++periapses >= 2 && first_sweep < 0.0) first_sweep = swept;
                swept = 0.0;
            }
            prev_vr = s.vr;
            const double dx = p[0] - last[0], dy = p[1] - last[1], dz = p[2] - last[2];
            if (sqrt(dx * dx + dy * dy + dz * dz) >= min_spacing && count < max_points) {
                if (pts) {
                    pts[3 * count] = p[0]; pts[3 * count + 1] = p[1]; pts[3 * count + 2] = p[2];
                }
                ++count;
                last[0] = p[0]; last[1] = p[1]; last[2] = p[2];
            }
        }
        ks_cartesian(a, s, p);  // the final position is always the path's last point
        if (pts) {
            pts[3 * count] = p[0]; pts[3 * count + 1] = p[1]; pts[3 * count + 2] = p[2];
        }
        ++count;
        if (out.fate) out.fate[i] = fate;
        if (out.duration) out.duration[i] = s.t - t0;
        if (out.r_min) out.r_min[i] = rmin;
        if (out.r_max) out.r_max[i] = rmax;
        if (out.periapses) out.periapses[i] = periapses;
        if (out.precession_deg) out.precession_deg[i] = first_sweep > 0.0 ? (first_sweep - 2.0 * kPi) * 180.0 / kPi : 0.0;
        if (out.n_points) out.n_points[i] = count;
        if (s_out) st(s, s_out[i]);
    }
}

}  // namespace

cudaError_t steps_predict(double a, const bhk_constants* c, const bhk_state* s, int64_t n, double max_time,
                          double min_spacing, int32_t max_points, double surface, double escape_radius,
                          bhk_state* s_out, const bhk_path_out& out, cudaStream_t st) {
    k_predict<<<grid_for(n), 64, 0, st>>>(a, c, s, n, max_time, min_spacing, max_points, surface, escape_radius,
                                          s_out, out);
    return cudaGetLastError();
}

cudaError_t steps_derivatives(double a, const bhk_constants* c, const bhk_state* s, bhk_derivatives_t* d, int64_t n,
                              cudaStream_t st) {
    k_derivatives<<<grid_for(n), kBlock, 0, st>>>(a, c, s, d, n);
    return cudaGetLastError();
}
cudaError_t steps_step_mino(double a, const bhk_constants* c, bhk_state* s, const double* h, int64_t n,
                            cudaStream_t st) {
    k_step_mino<<<grid_for(n), kBlock, 0, st>>>(a, c, s, h, n);
    return cudaGetLastError();
}
cudaError_t steps_photon_step_size(double a, const bhk_constants* c, const bhk_state* s, double tol, double* h,
                                   int64_t n, cudaStream_t st) {
    k_step_size<<<grid_for(n), kBlock, 0, st>>>(a, c, s, tol, h, n);
    return cudaGetLastError();
}
cudaError_t steps_enforce_constraints(double a, const bhk_constants* c, bhk_state* s, int64_t n, cudaStream_t st) {
    k_enforce<<<grid_for(n), kBlock, 0, st>>>(a, c, s, n);
    return cudaGetLastError();
}
cudaError_t steps_normalize_angles(bhk_state* s, int64_t n, cudaStream_t st) {
    k_normalize<<<grid_for(n), kBlock, 0, st>>>(s, n);
    return cudaGetLastError();
}
cudaError_t steps_potentials(double a, const bhk_constants* c, const bhk_state* s, double* R, double* Th, int64_t n,
                             cudaStream_t st) {
    k_potentials<<<grid_for(n), kBlock, 0, st>>>(a, c, s, R, Th, n);
    return cudaGetLastError();
}
cudaError_t steps_observer_frame(double a, const double* r, const double* th, const double* u, bhk_frame* f, int64_t n,
                                 cudaStream_t st) {
    k_frame<<<grid_for(n), kBlock, 0, st>>>(a, r, th, u, f, n);
    return cudaGetLastError();
}
cudaError_t steps_photon_from_frame(double a, double r, double th, double ph, const bhk_frame* f, const double* look,
                                    bhk_constants* c, bhk_state* s, int64_t n, cudaStream_t st) {
    k_photon<<<grid_for(n), kBlock, 0, st>>>(a, r, th, ph, f, look, c, s, n);
    return cudaGetLastError();
}
cudaError_t steps_launch_from_zamo(double a, double r, double th, double ph, const double* v, double mu,
                                   bhk_constants* c, bhk_state* s, int64_t n, cudaStream_t st) {
    k_zamo<<<grid_for(n), kBlock, 0, st>>>(a, r, th, ph, v, mu, c, s, n);
    return cudaGetLastError();
}
cudaError_t steps_cartesian_velocity(double a, const bhk_constants* c, const bhk_state* s, double* out, int64_t n,
                                     cudaStream_t st) {
    k_cartesian<<<grid_for(n), kBlock, 0, st>>>(a, c, s, out, n);
    return cudaGetLastError();
}

}  // namespace bhk
