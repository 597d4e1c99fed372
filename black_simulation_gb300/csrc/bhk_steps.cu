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

}  // namespace

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
