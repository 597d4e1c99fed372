// bhk_trace.cu -- the batch tracer for sm_103a.
//
// Pipeline of one batch (all on one stream, capturable as one CUDA graph):
//   frame_setup   1 block, FP64: per-frame ZAMO tetrad (kerr::observerFrame), its lowered vectors,
//                 horizon, ISCO, capture and escape radii
//   launch        FP64, one thread per ray: pinhole (alpha, beta) -> look -> kerr::photonFromFrame
//                 -> E, L, Q, vr, vtheta (the axis snap included); cost bucket. For frames traced
//                 without the cost sort the trace kernel does this itself as it takes the rays.
//   order         frames: by 8 x 4 pixel tiles, mapped in the trace kernel; or the cost sort: bucket
//                 histogram / scan / block-aggregated scatter, costliest first
//   trace         persistent grid; every lane owns one ray; a warp takes 32 queue-adjacent rays
//                 from the device queue and traces them to completion before it takes the next 32
//                 (rays that start together stay alike, so the warp's lanes take the same branches).
//                 Dormand-Prince 5(4) with FSAL and dense-output event location, in FP64 (parity
//                 mode) or FP32 (mixed mode: FP64 for the launch constants, the disk g, the analytic
//                 capture test near the horizon and the optional periodic radial re-projection)
//   rescue        FP64 continuation of the rare rays the FP32 kernel hands over
//
// The reference's ray semantics (src/trajectory.cpp:259-392): backward march in Mino time; disk
// where theta crosses pi/2 with r in [r_in, r_out] and g from prograde circular gas; captured when
// falling below r_+(1 + eps); escaped when rising past max(r_escape, 1.5 r_obs). Past |a| = 1 (no
// horizon) the renderer's rules (shaders/trace.frag:1768-1787): the ring singularity where
// Sigma < 4e-4, and the sky of the r < 0 region when falling past -max(r_escape, 1.5 r_obs).
#include "bhk_device.cuh"
#include "bhk_internal.h"

namespace bhk {

namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ double nan_d() { return __longlong_as_double(0x7ff8000000000000ULL); }

__device__ __forceinline__ double wrap_2pi(double x) {
    const double t = 2.0 * kPi;
    double y = x - t * floor(x / t);
    if (y >= t) y -= t;
    return y;
}

__host__ __device__ __forceinline__ RayGeom make_geom(double a, double r, double th, double ph, double r_in_opt,
                                                      double r_out, const TraceParams& p) {
    RayGeom g;
    g.a = a; g.r0 = r; g.th0 = th; g.ph0 = ph;
    g.rp = horizon_radius(a);
    g.r_cap = g.rp * (1.0 + p.eps);
    g.r_esc = fmax(p.r_escape, 1.5 * r);
    g.r_in = r_in_opt > 0.0 ? r_in_opt : isco_radius(a, true);
    g.r_out = r_out;
    // The analytic capture zone's top, never below the capture radius (a disk reaching inside r_+).
    g.zone_top = fmax(g.rp + dmind(0.05, 0.5 * (g.r_in - g.rp)), g.r_cap);
    g.naked = naked(a) ? 1 : 0;
    if (g.naked) {  // no horizon: nothing is captured (the ring and the far sky are tested instead)
        g.r_cap = -1e30;
        g.zone_top = -1e30;
    }
    // FP32 copies; the launch polar angle is stored relative to the camera's hemisphere (the FP32
    // tracer integrates pi - theta in the south).
    g.south0 = th > 0.5 * kPi ? 1 : 0;
    g.af = float(a); g.r0f = float(r); g.th0f = float(g.south0 ? kPi - th : th); g.ph0f = float(ph);
    g.r_capf = float(g.r_cap); g.r_escf = float(g.r_esc); g.r_inf = float(g.r_in); g.r_outf = float(g.r_out);
    g.zone_topf = float(g.zone_top); g.rpf = float(g.rp);
    g.dead = 0;
    g.pad = 0;
    return g;
}

// Cost bucket: photons whose b^2 + q sits near the critical value 27 wind near the photon orbit
// and take the most steps; bucket 0 holds them, so the queue serves the longest rays first.
__device__ __forceinline__ uint16_t cost_key(double E, double L, double Q, int buckets) {
    if (buckets <= 1) return 0;
    const float u = static_cast<float>((L * L + Q) / (E * E));
    const float d = fabsf(__logf(fmaxf(u, 1e-30f) * (1.0f / 27.0f)));
    const int k = static_cast<int>(d * buckets * (1.0f / 3.0f));
    return static_cast<uint16_t>(k < 0 ? 0 : (k >= buckets ? buckets - 1 : k));
}

// kerr::photonStepSize (src/kerr.cpp:563-575) from derivatives already evaluated, negated: the
// first step of the backward march. Lengths are r, or past |a| = 1 max(sqrt(Sigma), 0.02).
template <typename T>
__device__ __forceinline__ T first_step(const T y[5], const T k[5], T tol, T a2, bool nkd) {
    T sn, cs;
    Math<T>::sc(y[1], &sn, &cs);
    sn = fabs(sn);
    const T rs = nkd ? fmax(sqrt(y[0] * y[0] + a2 * cs * cs), T(0.02)) : y[0];
    const T t = tol * fmin(fmax(rs / T(8), T(1)), T(4));
    T h = t / (fabs(k[0]) / rs + fabs(k[1]) / fmax(sn, T(1e-4)) + fabs(k[2]) + T(1e-6));
    h = fmin(h, sqrt(t * rs / (fabs(k[3]) + T(1e-6))));
    h = fmin(h, sqrt(t * fmax(sn, T(1e-4)) / (fabs(k[4]) + T(1e-6))));
    return -h;
}

// The launch record of ray i. For FP32 runs also the FP32 tracer's start: the right-hand side at the
// launch point and the first step, from exactly the FP32 values the tracer starts from.
__device__ __forceinline__ void store_launch(LaunchSoA L, int64_t i, const RayGeom& g, double E, double Lz, double Q,
                                             double vr, double vth, int32_t gid, const TraceParams& p) {
    L.E[i] = E; L.L[i] = Lz; L.Q[i] = Q;
    L.vr[i] = vr; L.vth[i] = vth;
    L.geom_id[i] = gid;
    L.key[i] = cost_key(E, Lz, Q, p.buckets);
    const double x = Lz - g.a * E;
    const float4 cf = make_float4(float(E), float(Lz), float(Q), float(x * x + Q));
    const float2 vf = make_float2(float(vr), float(vth));
    L.cf[i] = cf;
    L.vf[i] = vf;
    if (L.kf) {
        RayC<float> c;
        c.set_t(g.af, cf.x, cf.y, cf.z, cf.w);
        const float y[5] = {g.r0f, g.th0f, g.ph0f, vf.x, g.south0 ? -vf.y : vf.y};
        float k[5];
        rhs(c, y, k);
        const float h = first_step<float>(y, k, p.tol0_f, c.a2, g.naked != 0);
        L.kf[i] = make_float4(k[0], k[1], k[2], k[3]);
        L.khf[i] = make_float2(k[4], h);
    }
}

// ------------------------------------------------------------------------- set-up kernels ----

// Per-frame set-up in FP64: the ZAMO tetrad at the camera (kerr::observerFrame), its vectors
// lowered with the camera's metric, the pieces of kerr::photonFromFrame that do not depend on the
// pixel, and the frame's ray geometry (horizon, ISCO, capture and escape radii). The API's batches
// do this on the host while staging the frame table; the allocation-free entry point on the device.
__host__ __device__ inline void setup_frame(FrameDev& fr, RayGeom& geom, const TraceParams& p) {
    const bhk_frame_desc d = fr.d;
    double u[4], e[4][4], g[4][4];
    zamo_four_velocity(d.a, d.r_obs, d.theta_obs, u);
    observer_frame(d.a, d.r_obs, d.theta_obs, u, e);
    metric_tensor(d.a, d.r_obs, d.theta_obs, g);
    for (int k = 0; k < 4; ++k)
        for (int i = 0; i < 4; ++i) {
            fr.e[k][i] = e[k][i];
            double acc = 0.0;
            for (int j = 0; j < 4; ++j) acc += g[i][j] * e[k][j];
            fr.el[k][i] = acc;
        }
    double sn, cs;
    sincos(d.theta_obs, &sn, &cs);
    fr.sigma = metric_at(d.a, d.r_obs, d.theta_obs).sigma;
    fr.cs2 = cs * cs;
    fr.inv_sn2 = 1.0 / dmaxd(sn * sn, 1e-18);
    fr.a2 = d.a * d.a;
    fr.inv_r = 1.0 / d.r_obs;
    fr.px = (d.alpha_hi - d.alpha_lo) / d.width;
    fr.py = (d.beta_hi - d.beta_lo) / d.height;
    geom = make_geom(d.a, d.r_obs, d.theta_obs, d.phi_obs, d.r_disk_in, d.r_disk_out, p);
}

__global__ void frame_setup_kernel(FrameDev* frames, RayGeom* geom, int nframes, TraceParams p, Control* ctl) {
    if (threadIdx.x == 0) {
        long long off = 0;
        for (int f = 0; f < nframes; ++f) {
            frames[f].offset = off;
            off += static_cast<long long>(frames[f].d.width) * frames[f].d.height;
        }
        ctl->n_rays = off;
    }
    for (int f = threadIdx.x; f < nframes; f += blockDim.x) setup_frame(frames[f], geom[f], p);
}

// 1/sqrt(x) in FP64 for x in [1, ~10]: FP32 seed (rsqrt.approx, ~2^-22 relative) refined by two Newton
// steps y <- y (3 - x y^2) / 2 (each squares the relative error): ~1 ulp without a DP divide or sqrt.
__device__ __forceinline__ double rsqrt_newton(double x) {
    float yf;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(yf) : "f"(static_cast<float>(x)));
    double y = yf;
    y = y * (1.5 - 0.5 * x * y * y);
    y = y * (1.5 - 0.5 * x * y * y);
    return y;
}

// kerr::photonFromFrame for pixel (alpha, beta) of a ZAMO pinhole, with the camera's metric
// contractions precomputed: p_mu = (g e_0)_mu - look^i (g e_i)_mu, p^r = e_0^r - look^i e_i^r.
// Launch record i for global pixel `pix` of the frame table (binary search over frame offsets).
struct Launched {
    double E, L, Q, vr, vth;
    int32_t gid;  // frame (geometry record) of the pixel
};

// The frame of global ray index i (binary search over the frame offsets).
__device__ __forceinline__ int frame_of(const FrameDev* __restrict__ frames, int nframes, long long i) {
    int lo = 0, hi = nframes - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (frames[mid].offset <= i) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// A warp's batch of 32 rays is an 8 x 4 tile of pixels (ragged at the right and bottom edges): queue
// position q of a W x H frame is pixel (x, y) with q = 4 ty W + hh 8 tx + (y - 4 ty) ww + (x - 8 tx),
// tile (tx, ty) = (x / 8, y / 4), hh and ww the tile's height and width. 8 wide rather than 4: the
// batch's results are written together, and each tile row is then a 64-byte run of every double
// output (for page-locked host outputs, 12 % more rays/s end to end on a 64-frame batch than with
// 4 x 8 tiles, at the same rays/s on the device).
constexpr int kTileW = 8, kTileH = 4;

__device__ __forceinline__ void tile_pixel(int W, int H, int lq, int* row, int* col) {
    const int ty = lq / (kTileH * W);
    const int rem = lq - ty * kTileH * W;
    const int hh = H - kTileH * ty < kTileH ? H - kTileH * ty : kTileH;
    const int tx = rem / (hh * kTileW);
    const int rem2 = rem - tx * hh * kTileW;
    const int ww = W - kTileW * tx < kTileW ? W - kTileW * tx : kTileW;
    const int dy = rem2 / ww;
    *row = kTileH * ty + dy;
    *col = kTileW * tx + (rem2 - dy * ww);
}

__device__ __forceinline__ Launched photon_at(const FrameDev& f, int fi, int row, int col) {
    const int lo = fi;
    const double alpha = f.d.alpha_lo + (col + 0.5) * f.px;
    const double beta = f.d.beta_hi - (row + 0.5) * f.py;
    const double lt = -beta * f.inv_r, lp = alpha * f.inv_r;
    const double inv = rsqrt_newton(1.0 + lt * lt + lp * lp);
    const double l0 = -inv, l1 = lt * inv, l2 = lp * inv;
    const double pt = f.el[0][0] - l0 * f.el[1][0] - l1 * f.el[2][0] - l2 * f.el[3][0];
    const double pth = f.el[0][2] - l0 * f.el[1][2] - l1 * f.el[2][2] - l2 * f.el[3][2];
    const double pph = f.el[0][3] - l0 * f.el[1][3] - l1 * f.el[2][3] - l2 * f.el[3][3];
    const double pr_up = f.e[0][1] - l0 * f.e[1][1] - l1 * f.e[2][1] - l2 * f.e[3][1];
    const double E = -pt;
    double Lz = pph;
    const double vr = f.sigma * pr_up;
    const double vth = pth;
    const double a2E2 = f.a2 * E * E;
    double Q = vth * vth + f.cs2 * (Lz * Lz * f.inv_sn2 - a2E2);
    // kAxisSnap (src/kerr.h:115): |L| < 3e-4 sqrt(Q + a^2 E^2), compared squared.
    if (Lz * Lz < 9e-8 * dmaxd(Q + a2E2, 0.0)) {
        Lz = 0.0;
        Q = vth * vth - f.cs2 * a2E2;
    }
    return Launched{E, Lz, Q, vr, vth, lo};
}

__device__ __forceinline__ Launched photon_of_pixel(const FrameDev* __restrict__ frames, int nframes, long long pix) {
    const int fi = frame_of(frames, nframes, pix);
    const FrameDev& f = frames[fi];
    const int local = static_cast<int>(pix - f.offset);  // < 2^31 rays per batch
    const int row = local / f.d.width;
    return photon_at(f, fi, row, local - row * f.d.width);
}

__device__ __forceinline__ void launch_pixel(const FrameDev* __restrict__ frames, const RayGeom* __restrict__ geom,
                                             int nframes, long long pix, long long i, LaunchSoA& L,
                                             const TraceParams& p) {
    const Launched x = photon_of_pixel(frames, nframes, pix);
    store_launch(L, i, geom[x.gid], x.E, x.L, x.Q, x.vr, x.vth, x.gid, p);
}

__global__ void launch_frames_kernel(const FrameDev* __restrict__ frames, const RayGeom* __restrict__ geom,
                                     int nframes, LaunchSoA L, TraceParams p, const Control* __restrict__ ctl) {
    const long long n = ctl->n_rays;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x)
        launch_pixel(frames, geom, nframes, i, i, L, p);
}

// Launch records for a list of global pixel indices (record i traces pixel list[i]).
__global__ void launch_list_kernel(const FrameDev* __restrict__ frames, const RayGeom* __restrict__ geom, int nframes,
                                   const int32_t* __restrict__ list, LaunchSoA L, TraceParams p,
                                   const Control* __restrict__ ctl) {
    const long long n = ctl->n_rays;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x)
        launch_pixel(frames, geom, nframes, list[i], i, L, p);
}

__global__ void launch_explicit_kernel(const double* __restrict__ a, const double* __restrict__ r_obs,
                                       const double* __restrict__ th_obs, const double* __restrict__ alpha,
                                       const double* __restrict__ beta, double r_in, double r_out, RayGeom* geom,
                                       LaunchSoA L, TraceParams p, const Control* __restrict__ ctl) {
    const long long n = ctl->n_rays;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const double ai = a[i], ri = r_obs[i], ti = th_obs[i];
        double u[4], e[4][4];
        zamo_four_velocity(ai, ri, ti, u);
        observer_frame(ai, ri, ti, u, e);
        const double lr = -1.0, lt = -beta[i] / ri, lp = alpha[i] / ri;
        const double nn = sqrt(lr * lr + lt * lt + lp * lp);
        const double look[3] = {lr / nn, lt / nn, lp / nn};
        Cons c;
        St s;
        photon_from_frame(ai, ri, ti, 0.0, e, look, c, s);
        const RayGeom g = make_geom(ai, ri, ti, 0.0, r_in, r_out, p);
        geom[i] = g;
        store_launch(L, i, g, c.E, c.L, c.Q, s.vr, s.vtheta, static_cast<int32_t>(i), p);
    }
}

// Launch records for cameras given by frame: trajectory::traceRay's launch (src/trajectory.cpp:
// 214-219) per ray, with its inside-horizon rule: a photon seen from inside the horizon with
// 2 r_+ E - a L < 0 came through the far side of the eternal spacetime (the hole) -- flagged dead.
__global__ void launch_framed_kernel(const double* __restrict__ a, const double* __restrict__ r,
                                     const double* __restrict__ th, const double* __restrict__ ph,
                                     const bhk_frame* __restrict__ frames, const double* __restrict__ look,
                                     double r_in, double r_out, RayGeom* geom, LaunchSoA L, TraceParams p,
                                     const Control* __restrict__ ctl) {
    const long long n = ctl->n_rays;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const double ai = a[i], ri = r[i], ti = th[i], pi = ph[i];
        double e[4][4];
        for (int k = 0; k < 4; ++k)
            for (int m = 0; m < 4; ++m) e[k][m] = frames[i].e[k][m];
        const double lk[3] = {look[3 * i], look[3 * i + 1], look[3 * i + 2]};
        Cons c;
        St s;
        photon_from_frame(ai, ri, ti, pi, e, lk, c, s);
        RayGeom g = make_geom(ai, ri, ti, pi, r_in, r_out, p);
        g.dead = (ri < g.rp && 2.0 * g.rp * c.E - ai * c.L < 0.0) ? 1 : 0;
        geom[i] = g;
        store_launch(L, i, g, c.E, c.L, c.Q, s.vr, s.vtheta, static_cast<int32_t>(i), p);
    }
}

// ----------------------------------------------------------------------------- pre-sort ----

__global__ void hist_kernel(LaunchSoA L, SortScratch S, TraceParams p, const Control* __restrict__ ctl) {
    __shared__ unsigned int h[kMaxBuckets];
    for (int b = threadIdx.x; b < p.buckets; b += blockDim.x) h[b] = 0;
    __syncthreads();
    const long long n = ctl->n_rays;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x)
        atomicAdd(&h[L.key[i]], 1u);
    __syncthreads();
    for (int b = threadIdx.x; b < p.buckets; b += blockDim.x)
        if (h[b]) atomicAdd(&S.hist[b], h[b]);
}

__global__ void scan_kernel(SortScratch S, TraceParams p) {
    if (threadIdx.x == 0) {
        unsigned int run = 0;
        for (int b = 0; b < p.buckets; ++b) {
            S.offs[b] = run;
            run += S.hist[b];
        }
    }
}

// Scatter in tiles of blockDim rays: ranks within a tile from shared-memory counters, one global
// atomic per (tile, bucket) to reserve the tile's slice of each bucket.
__global__ void scatter_kernel(LaunchSoA L, SortScratch S, TraceParams p, const Control* __restrict__ ctl) {
    __shared__ unsigned int cnt[kMaxBuckets];
    __shared__ unsigned int base[kMaxBuckets];
    const long long n = ctl->n_rays;
    const long long tiles = (n + blockDim.x - 1) / blockDim.x;
    for (long long t = blockIdx.x; t < tiles; t += gridDim.x) {
        for (int b = threadIdx.x; b < p.buckets; b += blockDim.x) cnt[b] = 0;
        __syncthreads();
        const long long i = t * blockDim.x + threadIdx.x;
        const bool live = i < n;
        const unsigned key = live ? L.key[i] : 0u;
        const unsigned rank = live ? atomicAdd(&cnt[key], 1u) : 0u;
        __syncthreads();
        for (int b = threadIdx.x; b < p.buckets; b += blockDim.x)
            if (cnt[b]) base[b] = atomicAdd(&S.offs[b], cnt[b]);
        __syncthreads();
        if (live) S.order[base[key] + rank] = static_cast<int32_t>(i);
        __syncthreads();
    }
}

// --------------------------------------------------------------------------- the tracer ----

enum : int { kContinue = 0, kFinished = 1, kRescue = 2, kRestart = 3 };

// float -> double by assembling the bits with integer operations: the FP32 tracer writes its double
// outputs without issuing conversions to the narrow FP64 pipe. Subnormal floats become zero.
__device__ __forceinline__ double f2d(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned sign = u & 0x80000000u;
    const unsigned e = (u >> 23) & 0xffu;
    const unsigned m = u & 0x7fffffu;
    unsigned hi;
    if (e == 0u) hi = sign;
    else if (e == 0xffu) hi = sign | 0x7ff00000u | (m >> 3) | (m ? 0x80000u : 0u);
    else hi = sign | ((e + 896u) << 20) | (m >> 3);
    return __hiloint2double(static_cast<int>(hi), static_cast<int>(m << 29));
}

__device__ __forceinline__ float nan_f() { return __int_as_float(0x7fc00000); }

// x wrapped to [0, 2 pi) in FP32: nearest multiple of 2 pi by the 1.5 * 2^23 rounding, removed with
// a two-constant split of 2 pi.
__device__ __forceinline__ float wrap_2pi_f(float x) {
    const float n = fmaf(x, 0.159154943091895336f, 12582912.0f) - 12582912.0f;
    float y = fmaf(n, -6.28318548202514648f, x);
    y = fmaf(n, 1.74845553e-7f, y);
    return y < 0.0f ? y + 6.28318548202514648f : y;
}

// disk_redshift in FP32 (src/trajectory.cpp:311-318): no cancellation at the disk radii.
__device__ __forceinline__ bool disk_redshift_f(float a, float E, float L, float rc, float* g) {
    const float irc = rcp_approx(rc);
    const float w = rcp_approx(rc * sqrt_approx(rc) + a);
    const float gtt = -(1.0f - 2.0f * irc), gtp = -2.0f * a * irc, gpp = rc * rc + a * a + 2.0f * a * a * irc;
    const float norm = -(gtt + 2.0f * gtp * w + gpp * w * w);
    if (!(norm > 0.0f)) return false;
    *g = sqrt_approx(norm) * rcp_approx(E - L * w);
    return true;
}

// FP32 tier of the capture test: no_radial_root_below with the bound required to clear FP32
// rounding by a wide margin (1e-4 of the polynomial's magnitude). False means "not proven": the
// FP64 test decides.
__device__ __forceinline__ bool no_radial_root_below_f(const RayC<float>& c, float x0, float r) {
    const float w = r - x0;
    if (w <= 0.0f) return true;
    const float xx = c.L - c.aE;
    const float c4 = c.E * c.E, c2 = -(2.0f * c.aE * xx + c.K), c1 = 2.0f * c.K, c0 = -c.a2 * c.Q;
    const float x2 = x0 * x0;
    const float R0 = ((c4 * x2 + c2) * x0 + c1) * x0 + c0;
    const float R1 = (4.0f * c4 * x2 + 2.0f * c2) * x0 + c1;
    const float R2 = 6.0f * c4 * x2 + c2;
    const float R3 = 4.0f * c4 * x0;
    const float lower = R0 - w * fmaxf(0.0f, -R1) - w * w * fmaxf(0.0f, -R2) - w * w * w * fmaxf(0.0f, -R3);
    const float scale = c4 * x2 * x2 + fabsf(c2) * x2 + fabsf(c1) * x0 + fabsf(c0);
    return lower > 1e-4f * scale;
}

template <typename T>
struct Lane {
    RayC<T> c;
    T y[5];
    T k[7][5];
    T h;
    T r_esc, zone_top;  // (the capture and disk radii are read from the geometry where they are needed)
    int acc, rej;
    // FP32 lanes: the outcome of a ray that has ended (-1 while it is traced). Its results wait in the
    // lane's state (y) and are written with the rest of the warp's batch by flush_f32: a warp's rays
    // end on different steps, and writing each as it ends runs that code once per step on which any
    // lane ended.
    int pend;
    bool last_rej;
    // FP32 only: the ray is in the southern hemisphere and y[1], y[4] hold pi - theta and -vtheta.
    // The Kerr metric is symmetric under theta -> pi - theta, so the equations are unchanged, and
    // both poles are approached with the full relative precision of a small angle.
    bool south;
    T rmin;          // closest approach so far (RayReport::rMin)
    // FP64 mode: Kerr-Schild time t as a passive extra component (its stage derivatives kt) and the
    // angle the position has swept (RayReport::delay, turns); `track` is false for FP32 lanes and for
    // the FP64 continuation of a mixed-precision ray, whose history is not known.
    bool track;
    double t, swept, kt[7], pos[3];
};

// Kerr-Schild Cartesian position (kerr::toCartesian, src/kerr.cpp:638-641).
__device__ __forceinline__ void ks_position(double a, double r, double th, double ph, double out[3]) {
    double st, ct, sp, cp;
    sincos(th, &st, &ct);
    sincos(ph, &sp, &cp);
    out[0] = (r * cp - a * sp) * st;
    out[1] = (r * sp + a * cp) * st;
    out[2] = r * ct;
}

template <typename T>
__device__ __forceinline__ void lane_radii(Lane<T>& s, const RayGeom& g) {
    if constexpr (sizeof(T) == 4) {
        s.r_esc = g.r_escf; s.zone_top = g.zone_topf;
    } else {
        s.r_esc = g.r_esc; s.zone_top = g.zone_top;
    }
}

// Starts an FP32 lane at its launch point from its launch record; the right-hand side there and the
// first step come prepared by the launch kernel when `have_k`, else are computed here.
__device__ __forceinline__ void lane_begin_f32(Lane<float>& s, const RayGeom& g, float4 cf, float2 vf, float4 k,
                                               float2 kh, bool have_k, const TraceParams& p) {
    s.c.set_t(g.af, cf.x, cf.y, cf.z, cf.w);
    s.south = g.south0 != 0;
    s.y[0] = g.r0f; s.y[1] = g.th0f; s.y[2] = g.ph0f; s.y[3] = vf.x; s.y[4] = s.south ? -vf.y : vf.y;
    lane_radii(s, g);
    s.rmin = s.y[0];
    s.t = 0.0;
    s.swept = 0.0;
    s.track = false;
    if (have_k) {
        s.k[0][0] = k.x; s.k[0][1] = k.y; s.k[0][2] = k.z; s.k[0][3] = k.w; s.k[0][4] = kh.x;
        s.h = kh.y;
    } else {
        rhs(s.c, s.y, s.k[0]);
        s.h = first_step<float>(s.y, s.k[0], p.tol0_f, s.c.a2, g.naked != 0);
    }
    s.acc = 0; s.rej = 0; s.last_rej = false; s.pend = -1;
}

// Starts an FP64 lane on ray `ray` at its launch point, first step from kerr::photonStepSize (the
// FP32 tracer starts its lanes with lane_begin_f32).
__device__ __forceinline__ void lane_begin_launch(Lane<double>& s, const RayGeom& g, const LaunchSoA& L, long long ray,
                                                  const TraceParams& p) {
    s.c.set(g.a, L.E[ray], L.L[ray], L.Q[ray]);
    s.south = false;
    s.y[0] = g.r0; s.y[1] = g.th0; s.y[2] = g.ph0; s.y[3] = L.vr[ray]; s.y[4] = L.vth[ray];
    lane_radii(s, g);
    s.rmin = s.y[0];
    s.t = 0.0;
    s.swept = 0.0;
    s.track = true;
    rhs(s.c, s.y, s.k[0], static_cast<Proj<double>*>(nullptr), &s.kt[0]);
    ks_position(g.a, s.y[0], s.y[1], s.y[2], s.pos);
    s.h = first_step<double>(s.y, s.k[0], p.tol0, s.c.a2, g.naked != 0);
    s.acc = 0; s.rej = 0; s.last_rej = false; s.pend = -1;
}

__device__ __forceinline__ void write_out(const Outputs& o, long long ray, int outcome, double rd, double pd, double g,
                                          double ti, double pi, int steps, int rejected) {
    if (o.outcome) o.outcome[ray] = static_cast<uint8_t>(outcome);
    if (o.r_disk) o.r_disk[ray] = rd;
    if (o.phi_disk) o.phi_disk[ray] = pd;
    if (o.g) o.g[ray] = g;
    if (o.theta_inf) o.theta_inf[ray] = ti;
    if (o.phi_inf) o.phi_inf[ray] = pi;
    if (o.steps) o.steps[ray] = steps;
    if (o.rejected) o.rejected[ray] = rejected;
}

template <typename T>
__device__ __forceinline__ void write_out_t(const Outputs& o, long long ray, int outcome, T rd, T pd, T g, T ti, T pi,
                                            int steps, int rejected) {
    if constexpr (sizeof(T) == 4) write_out(o, ray, outcome, f2d(rd), f2d(pd), f2d(g), f2d(ti), f2d(pi), steps, rejected);
    else write_out(o, ray, outcome, rd, pd, g, ti, pi, steps, rejected);
}

template <typename T>
__device__ __forceinline__ T nan_t() {
    if constexpr (sizeof(T) == 4) return nan_f();
    else return nan_d();
}

// The path outputs of a finished ray: closest approach (r_+(1 + eps) once captured), and in FP64 mode
// the time the light travelled (t runs backward from 0 at the camera) and the turns swept.
template <typename T>
__device__ __forceinline__ void write_path(const Lane<T>& s, const Outputs& o, long long ray, double t_end,
                                           double r_cap = INFINITY) {
    if (o.r_min) o.r_min[ray] = fmin(double(s.rmin), r_cap);
    if (o.delay) o.delay[ray] = s.track ? -t_end : nan_d();
    if (o.turns) o.turns[ray] = s.track ? s.swept / (2.0 * kPi) : nan_d();
}

// A ray that ends without a disk or sky result. r_cap: the capture radius of a captured ray (its
// closest approach is at most that; FP32 lanes read it again when their batch is written).
template <typename T>
__device__ __forceinline__ int finish(Lane<T>& s, const Outputs& o, long long ray, int outcome, Control* ctl,
                                      double r_cap = INFINITY) {
    if constexpr (sizeof(T) == 4) {
        s.pend = outcome;
    } else {
        const T n = nan_t<T>();
        write_out_t<T>(o, ray, outcome, n, n, n, n, n, s.acc, s.rej);
        write_path(s, o, ray, s.t, r_cap);
        if (outcome == BHK_RAY_UNFINISHED) atomicAdd(&ctl->stats[2], 1ull);
    }
    return kFinished;
}

// Fraction of the step where the dense output of component i equals target: Newton on the quartic
// continuous extension from linear interpolation, kept inside the sign-change bracket [lo, hi]
// (bisection whenever Newton leaves it), until the step in s falls below the type's resolution.
template <typename T>
__device__ __forceinline__ T locate(const T* y0, const T* y1, const T k[7][5], T h, int i, T target) {
    constexpr int iters = sizeof(T) == 8 ? 64 : 32;
    constexpr T tiny = sizeof(T) == 8 ? T(1e-15) : T(1e-7);
    const T yd = y1[i] - y0[i];
    const T b = h * k[0][i] - yd;
    const T c4 = yd - h * k[6][i] - b;
    const T c5 = h * (T(DP::d1) * k[0][i] + T(DP::d3) * k[2][i] + T(DP::d4) * k[3][i] + T(DP::d5) * k[4][i] +
                      T(DP::d6) * k[5][i] + T(DP::d7) * k[6][i]);
    const T f0 = y0[i] - target;
    const bool neg0 = f0 < T(0);
    T lo = T(0), hi = T(1);
    T s = fmin(fmax(-f0 / yd, T(0)), T(1));
    for (int it = 0; it < iters; ++it) {
        const T s1 = T(1) - s;
        const T u = b + s * (c4 + s1 * c5);
        const T du = c4 + (T(1) - T(2) * s) * c5;
        const T w = yd + s1 * u;
        const T dw = -u + s1 * du;
        const T f = f0 + s * w;
        const T df = w + s * dw;
        if (f == T(0)) break;
        if ((f < T(0)) == neg0) lo = s; else hi = s;
        T sn = s - f / df;
        if (!(sn > lo && sn < hi)) sn = T(0.5) * (lo + hi);
        const bool done = fabs(sn - s) <= tiny || hi - lo <= tiny;
        s = sn;
        if (done) break;
    }
    return s;
}

// The escape direction at the exit point x (the state in the lane's hemisphere representation):
// the backward tangent there, as (theta_inf, phi_inf).
template <typename T>
__device__ __forceinline__ void exit_direction(const RayC<T>& c, bool south, const T x_in[5], T* theta_inf,
                                               T* phi_inf) {
    T x[5], kk[5];
#pragma unroll
    for (int i = 0; i < 5; ++i) x[i] = x_in[i];
    rhs(c, x, kk);
    T v[3];
    if (south) {  // back to the physical angle: cos(pi - t) = -cos t, d(pi - t) = -dt
        x[1] = T(kPi) - x[1];
        x[4] = -x[4];
    }
    cartesian_velocity<T>(c.a, x[0], x[1], x[2], x[3], x[4], kk[2], v);
    const T nrm = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    const T dz = fmin(fmax(-v[2] / nrm, T(-1)), T(1));
    *theta_inf = acos(dz);
    *phi_inf = atan2(-v[1] / nrm, -v[0] / nrm);
}

// A ray that left through r = target within the step just taken: the exit point from the dense
// output. FP32 lanes keep it in y and work out the direction when their batch is written.
template <typename T>
__device__ __forceinline__ int escape(Lane<T>& s, const T prev[5], T h, T target, int outcome, const Outputs& out,
                                   long long ray, double t_prev) {
    const T sg = locate(prev, s.y, s.k, h, 0, target);
    T x[5];
#pragma unroll
    for (int i = 0; i < 5; ++i) x[i] = dense(prev[i], s.y[i], s.k, h, i, sg);
    if constexpr (sizeof(T) == 4) {
#pragma unroll
        for (int i = 0; i < 5; ++i) s.y[i] = x[i];
        s.pend = outcome;
    } else {
        T ti, pi;
        exit_direction(s.c, s.south, x, &ti, &pi);
        const T n = nan_t<T>();
        write_out_t<T>(out, ray, outcome, n, n, n, ti, pi, s.acc, s.rej);
        write_path(s, out, ray, dense1(t_prev, s.t, s.kt, h, sg));
    }
    return kFinished;
}

// Writes the results of an FP32 lane whose ray has ended (s.pend): disk r, g, phi in y[0..2], the
// exit point in y for the skies; r_min, the steps and the capture radius as in finish().
__device__ __forceinline__ void flush_f32(const Lane<float>& s, const Outputs& o, long long ray, Control* ctl,
                                          const RayGeom* __restrict__ geom, const LaunchSoA& L) {
    const float n = nan_f();
    float rd = n, pd = n, g = n, ti = n, pi = n;
    double r_cap = INFINITY;
    const int oc = s.pend;
    if (oc == BHK_RAY_DISK) {
        rd = s.y[0]; g = s.y[1]; pd = s.y[2];
    } else if (oc == BHK_RAY_ESCAPED || oc == BHK_RAY_ESCAPED_BEYOND) {
        exit_direction(s.c, s.south, s.y, &ti, &pi);
    } else if (oc == BHK_RAY_CAPTURED) {
        r_cap = geom[L.geom_id[ray]].r_cap;
    } else if (oc == BHK_RAY_UNFINISHED) {
        atomicAdd(&ctl->stats[2], 1ull);
    }
    write_out_t<float>(o, ray, oc, rd, pd, g, ti, pi, s.acc, s.rej);
    write_path(s, o, ray, 0.0, r_cap);
}

// ---- packed FP32 (f32x2) pieces of the FP32 step ----
// The state's components pair up as (r, theta) = (0, 1) and (vr, vtheta) = (3, 4), with phi (2) alone;
// the pairs go through Blackwell's packed FP32 instructions, which do two lanes' worth of FP32 work per
// issued instruction (the tracer is bound by instruction issue, not by the FMA pipe).
__device__ __forceinline__ float2 pr01(const float v[5]) { return make_float2(v[0], v[1]); }
__device__ __forceinline__ float2 pr34(const float v[5]) { return make_float2(v[3], v[4]); }

// The Dormand-Prince coefficients the FP32 step multiplies, by position: [0, 20) the stage rows
// a21; a31 a32; ...; a61 .. a65 and the solution row b1 b3 b4 b5 b6, [20, 26) the error row
// e1 e3 e4 e5 e6 e7. Each enters a packed instruction as a pair (c, c), made from an immediate.
__device__ __forceinline__ constexpr float dp_coef(int i) {
    constexpr double c[26] = {DP::a21, DP::a31, DP::a32, DP::a41, DP::a42, DP::a43, DP::a51, DP::a52, DP::a53,
                              DP::a54, DP::a61, DP::a62, DP::a63, DP::a64, DP::a65, DP::b1,  DP::b3,  DP::b4,
                              DP::b5,  DP::b6,  DP::e1,  DP::e3,  DP::e4,  DP::e5,  DP::e6,  DP::e7};
    return float(c[i]);
}
constexpr int kCoefE = 20;
__device__ __forceinline__ float2 dp_pair(int i) { return make_float2(dp_coef(i), dp_coef(i)); }

// t = y + h sum_m a_m k[j_m] with a_m = dp_coef(O + m): the tableau row's sum first (a chain of fused
// multiply-adds in the order of m, from a product), then one fused multiply-add by h onto y.
template <int O, int M>
__device__ __forceinline__ void stage_f32(const float y[5], const float k[7][5], float2 hh, const int (&j)[M],
                                          float t[5]) {
    float2 u0 = __fmul2_rn(dp_pair(O), pr01(k[j[0]]));
    float2 u1 = __fmul2_rn(dp_pair(O), pr34(k[j[0]]));
    float u2 = __fmul_rn(dp_coef(O), k[j[0]][2]);
#pragma unroll
    for (int m = 1; m < M; ++m) {
        const float2 am = dp_pair(O + m);
        u0 = __ffma2_rn(am, pr01(k[j[m]]), u0);
        u1 = __ffma2_rn(am, pr34(k[j[m]]), u1);
        u2 = fmaf(am.x, k[j[m]][2], u2);
    }
    const float2 p0 = __ffma2_rn(hh, u0, pr01(y)), p1 = __ffma2_rn(hh, u1, pr34(y));
    t[0] = p0.x; t[1] = p0.y; t[2] = fmaf(hh.x, u2, y[2]); t[3] = p1.x; t[4] = p1.y;
}

// Sum over the components of (e_i / sc_i)^2, e = the embedded error estimate without its factor h and
// sc_i = rtol (1 + max(|y_i|, |y5_i|)): the FP32 error norm's sum, in the scalar form's rounding.
__device__ __forceinline__ float error_norm2_f32(const float y[5], const float y5[5], const float k[7][5], float rtol) {
    const float2 e1 = dp_pair(kCoefE), e3 = dp_pair(kCoefE + 1), e4 = dp_pair(kCoefE + 2), e5 = dp_pair(kCoefE + 3),
                 e6 = dp_pair(kCoefE + 4), e7 = dp_pair(kCoefE + 5);
    const float2 rt = make_float2(rtol, rtol);
    float2 q[2];
    float q2;
#pragma unroll
    for (int pr = 0; pr < 2; ++pr) {
        const int i = pr == 0 ? 0 : 3;
        const float2 k0 = make_float2(k[0][i], k[0][i + 1]), k2 = make_float2(k[2][i], k[2][i + 1]),
                     k3 = make_float2(k[3][i], k[3][i + 1]), k4 = make_float2(k[4][i], k[4][i + 1]),
                     k5 = make_float2(k[5][i], k[5][i + 1]), k6 = make_float2(k[6][i], k[6][i + 1]);
        float2 e = __fmul2_rn(e1, k0);
        e = __ffma2_rn(e3, k2, e);
        e = __ffma2_rn(e4, k3, e);
        e = __ffma2_rn(e5, k4, e);
        e = __ffma2_rn(e6, k5, e);
        e = __ffma2_rn(e7, k6, e);
        const float2 mx = make_float2(fmaxf(fabsf(y[i]), fabsf(y5[i])), fmaxf(fabsf(y[i + 1]), fabsf(y5[i + 1])));
        const float2 sc = __ffma2_rn(rt, mx, rt);
        q[pr] = __fmul2_rn(e, make_float2(rcp_approx(sc.x), rcp_approx(sc.y)));
    }
    {
        float e = __fmul_rn(e1.x, k[0][2]);
        e = fmaf(e3.x, k[2][2], e);
        e = fmaf(e4.x, k[3][2], e);
        e = fmaf(e5.x, k[4][2], e);
        e = fmaf(e6.x, k[5][2], e);
        e = fmaf(e7.x, k[6][2], e);
        const float sc = fmaf(rtol, fmaxf(fabsf(y[2]), fabsf(y5[2])), rtol);
        q2 = __fmul_rn(e, rcp_approx(sc));
    }
    // The sum in component order 0 .. 4, as the scalar loop accumulates it.
    float acc = __fmul_rn(q[0].x, q[0].x);
    acc = fmaf(q[0].y, q[0].y, acc);
    acc = fmaf(q2, q2, acc);
    acc = fmaf(q[1].x, q[1].x, acc);
    acc = fmaf(q[1].y, q[1].y, acc);
    return acc;
}

// A ray within ~0.05 M of a radial turning point (R ~ R'(r_t) (r - r_t), so |r - r_t| ~ vr^2 / |R'| with
// R' = 2 k[3]) or within ~0.05 rad of a polar one (the same with Theta and k[4]).
__device__ __forceinline__ bool near_turning_point(const Lane<float>& s) {
    return s.y[3] * s.y[3] < 0.1f * fabsf(s.k[0][3]) || s.y[4] * s.y[4] < 0.1f * fabsf(s.k[0][4]);
}

// The Dormand-Prince attempt of an FP32 lane taken in FP64: the right-hand side at the step's start
// (fresh, from the FP64 launch constants), the six stages, the 5th-order solution y5 and its
// constraint potentials, and the error estimate -- the arithmetic of the FP64 tracer, on the lane's
// hemisphere representation (the equations are symmetric under theta -> pi - theta). The stages and
// y5 go back to the lane as FP32, so that the step's events, acceptance, re-projection and step control
// stay the FP32 code's. Returns the squared error norm in the FP32 step's convention.
__device__ __noinline__ float attempt_stages_f64(const float y[5], float k[7][5], float h, double rtol, double a,
                                                 double E, double Lz, double Q, float y5[5], Proj<float>* pj) {
    RayC<double> c;
    c.set(a, E, Lz, Q);
    double yd[5], kd[7][5], t[5], y5d[5];
#pragma unroll
    for (int i = 0; i < 5; ++i) yd[i] = y[i];
    const double hd = h;
    rhs(c, yd, kd[0]);
#pragma unroll
    for (int i = 0; i < 5; ++i) t[i] = yd[i] + hd * (DP::a21 * kd[0][i]);
    rhs(c, t, kd[1]);
#pragma unroll
    for (int i = 0; i < 5; ++i) t[i] = yd[i] + hd * (DP::a31 * kd[0][i] + DP::a32 * kd[1][i]);
    rhs(c, t, kd[2]);
#pragma unroll
    for (int i = 0; i < 5; ++i) t[i] = yd[i] + hd * (DP::a41 * kd[0][i] + DP::a42 * kd[1][i] + DP::a43 * kd[2][i]);
    rhs(c, t, kd[3]);
#pragma unroll
    for (int i = 0; i < 5; ++i)
        t[i] = yd[i] + hd * (DP::a51 * kd[0][i] + DP::a52 * kd[1][i] + DP::a53 * kd[2][i] + DP::a54 * kd[3][i]);
    rhs(c, t, kd[4]);
#pragma unroll
    for (int i = 0; i < 5; ++i)
        t[i] = yd[i] + hd * (DP::a61 * kd[0][i] + DP::a62 * kd[1][i] + DP::a63 * kd[2][i] + DP::a64 * kd[3][i] +
                             DP::a65 * kd[4][i]);
    rhs(c, t, kd[5]);
#pragma unroll
    for (int i = 0; i < 5; ++i)
        y5d[i] = yd[i] + hd * (DP::b1 * kd[0][i] + DP::b3 * kd[2][i] + DP::b4 * kd[3][i] + DP::b5 * kd[4][i] +
                               DP::b6 * kd[5][i]);
    Proj<double> pd;
    rhs<double, true>(c, y5d, kd[6], &pd);
    double acc = 0.0;
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        const double e = DP::e1 * kd[0][i] + DP::e3 * kd[2][i] + DP::e4 * kd[3][i] + DP::e5 * kd[4][i] +
                         DP::e6 * kd[5][i] + DP::e7 * kd[6][i];
        const double q = e / (rtol + rtol * fmax(fabs(yd[i]), fabs(y5d[i])));
        acc += q * q;
    }
#pragma unroll
    for (int j = 0; j < 7; ++j)
#pragma unroll
        for (int i = 0; i < 5; ++i) k[j][i] = static_cast<float>(kd[j][i]);
#pragma unroll
    for (int i = 0; i < 5; ++i) y5[i] = static_cast<float>(y5d[i]);
    pj->R = static_cast<float>(pd.R);
    pj->Rz = static_cast<float>(pd.Rz);
    pj->Th = static_cast<float>(pd.Th);
    pj->Thz = static_cast<float>(pd.Thz);
    return static_cast<float>(acc * 0.2 * hd * hd);
}

// One Dormand-Prince attempt on a lane's ray. Returns kContinue, kFinished (outputs written),
// kRescue (FP32 only: hand the state to FP64) or kRestart (FP32 only: non-finite state).
// kTP (FP32 only): attempts that start near a turning point are taken in FP64 (attempt_stages_f64);
// n_tp counts them.
template <typename T, bool kTP = false>
__device__ __forceinline__ int attempt(Lane<T>& s, const TraceParams& p, long long ray, const Outputs& out,
                                       bool reproject, Control* ctl, const LaunchSoA& L,
                                       const RayGeom* __restrict__ geom, unsigned* n_tp = nullptr) {
    constexpr bool F64 = sizeof(T) == 8;
    const T h = s.h;
    T t[5];
    T y5[5];
    bool tp_step = false;
    if constexpr (!F64 && kTP) tp_step = near_turning_point(s);
    if (tp_step) {
        // (FP32 lanes only; the stages, y5, the FSAL stage's potentials and the error norm come below)
    } else if constexpr (F64) {  // the oracle's operation order
#pragma unroll
        for (int i = 0; i < 5; ++i) t[i] = s.y[i] + h * (T(DP::a21) * s.k[0][i]);
        rhs(s.c, t, s.k[1], static_cast<Proj<T>*>(nullptr), &s.kt[1]);
#pragma unroll
        for (int i = 0; i < 5; ++i) t[i] = s.y[i] + h * (T(DP::a31) * s.k[0][i] + T(DP::a32) * s.k[1][i]);
        rhs(s.c, t, s.k[2], static_cast<Proj<T>*>(nullptr), &s.kt[2]);
#pragma unroll
        for (int i = 0; i < 5; ++i)
            t[i] = s.y[i] + h * (T(DP::a41) * s.k[0][i] + T(DP::a42) * s.k[1][i] + T(DP::a43) * s.k[2][i]);
        rhs(s.c, t, s.k[3], static_cast<Proj<T>*>(nullptr), &s.kt[3]);
#pragma unroll
        for (int i = 0; i < 5; ++i)
            t[i] = s.y[i] + h * (T(DP::a51) * s.k[0][i] + T(DP::a52) * s.k[1][i] + T(DP::a53) * s.k[2][i] +
                                 T(DP::a54) * s.k[3][i]);
        rhs(s.c, t, s.k[4], static_cast<Proj<T>*>(nullptr), &s.kt[4]);
#pragma unroll
        for (int i = 0; i < 5; ++i)
            t[i] = s.y[i] + h * (T(DP::a61) * s.k[0][i] + T(DP::a62) * s.k[1][i] + T(DP::a63) * s.k[2][i] +
                                 T(DP::a64) * s.k[3][i] + T(DP::a65) * s.k[4][i]);
        rhs(s.c, t, s.k[5], static_cast<Proj<T>*>(nullptr), &s.kt[5]);
#pragma unroll
        for (int i = 0; i < 5; ++i)
            y5[i] = s.y[i] + h * (T(DP::b1) * s.k[0][i] + T(DP::b3) * s.k[2][i] + T(DP::b4) * s.k[3][i] +
                                  T(DP::b5) * s.k[4][i] + T(DP::b6) * s.k[5][i]);
    } else {
        // FP32: each stage's sum y + h sum_j a_ij k_j with the pairs (r, theta) and (vr, vtheta) on
        // the packed f32x2 instructions (two components per instruction), phi alone.
        const float2 hh = make_float2(h, h);
        stage_f32<0, 1>(s.y, s.k, hh, {0}, t);
        rhs(s.c, t, s.k[1]);
        stage_f32<1, 2>(s.y, s.k, hh, {0, 1}, t);
        rhs(s.c, t, s.k[2]);
        stage_f32<3, 3>(s.y, s.k, hh, {0, 1, 2}, t);
        rhs(s.c, t, s.k[3]);
        stage_f32<6, 4>(s.y, s.k, hh, {0, 1, 2, 3}, t);
        rhs(s.c, t, s.k[4]);
        stage_f32<10, 5>(s.y, s.k, hh, {0, 1, 2, 3, 4}, t);
        rhs(s.c, t, s.k[5]);
        stage_f32<15, 5>(s.y, s.k, hh, {0, 2, 3, 4, 5}, y5);
    }
    Proj<T> pj;
    float tp_e2 = 0.0f;
    if constexpr (F64) {
        rhs<T, false>(s.c, y5, s.k[6], &pj, &s.kt[6]);
    } else {
        if (tp_step) {
            if constexpr (kTP) {
                const RayGeom& G = geom[L.geom_id[ray]];
                tp_e2 = attempt_stages_f64(s.y, s.k, h, p.rtol, G.a, L.E[ray], L.L[ray], L.Q[ray], y5, &pj);
                ++*n_tp;
            }
        } else {
            rhs<T, true>(s.c, y5, s.k[6], &pj);
        }
    }
    T rtol;
    if constexpr (F64) rtol = p.rtol;
    else rtol = p.rtol_f;
    T acc = T(0);
    if constexpr (F64) {
#pragma unroll
        for (int i = 0; i < 5; ++i) {
            const T e = h * (T(DP::e1) * s.k[0][i] + T(DP::e3) * s.k[2][i] + T(DP::e4) * s.k[3][i] +
                             T(DP::e5) * s.k[4][i] + T(DP::e6) * s.k[5][i] + T(DP::e7) * s.k[6][i]);
            const T sc = rtol + rtol * fmax(fabs(s.y[i]), fabs(y5[i]));
            const T q = Math<T>::div(e, sc);
            acc += q * q;
        }
    } else {
        if (!tp_step) acc = error_norm2_f32(s.y, y5, s.k, rtol);  // without the factor h, applied once below
    }
    // err = sqrt(acc / 5); the FP32 path works with err^2.
    T err, e2;
    bool ok;
    if constexpr (F64) {
        err = sqrt(acc / T(5));
        e2 = err;
        ok = err <= T(1);
    } else {
        e2 = tp_step ? tp_e2 : acc * (T(0.2) * h * h);
        err = e2;
        ok = e2 <= T(1);
    }
    if (!ok) {
        ++s.rej;
        s.last_rej = true;
        T fac;
        if constexpr (F64) fac = isfinite(err) ? fmax(0.2, 0.9 * pow(err, -0.2)) : 0.2;
        else fac = isfinite(e2) ? fmaxf(0.2f, 0.9f * exp2f(-0.1f * __log2f(e2))) : 0.2f;
        s.h = h * fac;
        if (s.rej >= p.max_steps) return finish(s, out, ray, BHK_RAY_UNFINISHED, ctl);
        return kContinue;
    }
    ++s.acc;
    T prev[5];
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        prev[i] = s.y[i];
        s.y[i] = y5[i];
    }
    if constexpr (F64) {
        if (!isfinite(s.y[0])) return finish(s, out, ray, BHK_RAY_UNFINISHED, ctl);
    }
    // Closest approach (when asked for): the step's end, or inside it where vr changes sign (the
    // turning point, from the dense output).
    if (out.r_min) {
        if (prev[3] * s.y[3] < T(0)) {
            const T sv = locate(prev, s.y, s.k, h, 3, T(0));
            s.rmin = fmin(s.rmin, dense(prev[0], s.y[0], s.k, h, 0, sv));
        }
        s.rmin = fmin(s.rmin, s.y[0]);
    }
    double t_prev = 0.0;
    if constexpr (F64) {
        t_prev = s.t;
        s.t += h * (DP::b1 * s.kt[0] + DP::b3 * s.kt[2] + DP::b4 * s.kt[3] + DP::b5 * s.kt[4] + DP::b6 * s.kt[5]);
        // The angle swept between the step's ends, as trajectory::traceRay sums it (src/trajectory.cpp:299).
        double x1[3];
        ks_position(s.c.a, s.y[0], s.y[1], s.y[2], x1);
        const double n0 = sqrt(s.pos[0] * s.pos[0] + s.pos[1] * s.pos[1] + s.pos[2] * s.pos[2]);
        const double n1 = sqrt(x1[0] * x1[0] + x1[1] * x1[1] + x1[2] * x1[2]);
        const double cang = (s.pos[0] * x1[0] + s.pos[1] * x1[1] + s.pos[2] * x1[2]) / fmax(n0 * n1, 1e-300);
        s.swept += acos(fmin(fmax(cang, -1.0), 1.0));
        s.pos[0] = x1[0]; s.pos[1] = x1[1]; s.pos[2] = x1[2];
    }
    const bool falling = s.y[0] < prev[0];
    // The rare events of a step, tested at once for FP32 lanes: a non-finite state, the ring's
    // neighbourhood, escape, the capture zone, a pole or the equator crossed (a disk crossing is one)
    // and the step limit. Most steps meet none and pass all of their code with one branch.
    bool rare = true;
    if constexpr (!F64) {
        const T a0 = fabs(s.y[0]);
        rare = !(a0 >= T(0.02) && a0 <= s.r_esc) || (s.y[0] < s.zone_top && falling) || s.y[1] < T(0) ||
               s.y[1] > T(0.5 * kPi) || s.acc >= p.max_steps;
    }
    if (rare) {
        if constexpr (!F64) {
            if (!isfinite(s.y[0])) return kRestart;
        }
        const T hp = T(0.5 * kPi);
        // Thin disk: theta crosses pi/2 inside [r_in, r_out]. (FP32: the hemisphere representation keeps
        // theta at or below pi/2 at a step's start, so a crossing is theta above pi/2 at its end.)
        bool crossed;
        if constexpr (F64) crossed = (prev[1] - hp) * (s.y[1] - hp) < T(0);
        else crossed = prev[1] < hp && s.y[1] > hp;
        if (crossed) {
            const T sg = locate(prev, s.y, s.k, h, 1, hp);
            const T rc = dense(prev[0], s.y[0], s.k, h, 0, sg);
            const RayGeom& G = geom[L.geom_id[ray]];
            T r_in, r_out;
            if constexpr (F64) { r_in = G.r_in; r_out = G.r_out; } else { r_in = G.r_inf; r_out = G.r_outf; }
            if (rc >= r_in && rc <= r_out) {
                if constexpr (F64) {
                    double g;
                    if (disk_redshift(s.c.a, s.c.E, s.c.L, rc, &g)) {
                        const double ph = wrap_2pi(dense(prev[2], s.y[2], s.k, h, 2, sg));
                        write_out(out, ray, BHK_RAY_DISK, rc, ph, g, nan_d(), nan_d(), s.acc, s.rej);
                        write_path(s, out, ray, dense1(t_prev, s.t, s.kt, h, sg));
                        return kFinished;
                    }
                } else {
                    float g;
                    if (disk_redshift_f(s.c.a, s.c.E, s.c.L, rc, &g)) {
                        const float ph = wrap_2pi_f(dense(prev[2], s.y[2], s.k, h, 2, sg));
                        s.y[0] = rc; s.y[1] = g; s.y[2] = ph;  // written with the batch (flush_f32)
                        s.pend = BHK_RAY_DISK;
                        return kFinished;
                    }
                }
            }
        }
        // Past |a| = 1 only (around a hole r stays above r_+ > 1): the ring singularity, where
        // Sigma = r^2 + a^2 cos^2(theta) < 4e-4 (shaders/trace.frag:1773-1778). That needs |r| < 0.02 and
        // |cos theta| < 0.02 / |a|, where cos theta = sin d, d = pi/2 - theta, is d - d^3/6 to 3e-11 (the
        // same in either hemisphere representation).
        if (fabs(s.y[0]) < T(0.02)) {
            const T d = T(0.5 * kPi) - s.y[1];
            const T c = d - d * d * d * T(1.0 / 6.0);
            if (s.y[0] * s.y[0] + s.c.a2 * c * c < T(4e-4)) return finish(s, out, ray, BHK_RAY_RING, ctl);
        }
        // Escaped: rising past r_esc, or past |a| = 1 falling past -r_esc into the sky of the r < 0 region,
        // beyond the ring (shaders/trace.frag:1779-1792). Rays start inside |r| < r_esc (the camera sits
        // within r_esc / 1.5), so |r| first exceeds r_esc on the step that leaves.
        if (fabs(s.y[0]) > s.r_esc) {
            const bool beyond = s.y[0] < T(0);
            return escape(s, prev, h, beyond ? -s.r_esc : s.r_esc,
                          beyond ? BHK_RAY_ESCAPED_BEYOND : BHK_RAY_ESCAPED, out, ray, t_prev);
        }
        // Captured (zone_top lies above r_cap; both are -1e30 past |a| = 1; r_cap is read from the
        // geometry here rather than held in a register).
        if (s.y[0] < s.zone_top && falling) {
            const RayGeom& G = geom[L.geom_id[ray]];
            if (s.y[0] < (F64 ? T(G.r_cap) : T(G.r_capf))) return finish(s, out, ray, BHK_RAY_CAPTURED, ctl, G.r_cap);
            if constexpr (F64) {
                if (no_radial_root_below(s.c.a, s.c.E, s.c.L, s.c.Q, s.y[0], p.eps))
                    return finish(s, out, ray, BHK_RAY_CAPTURED, ctl, G.r_cap);
            } else {
                if (no_radial_root_below_f(s.c, G.r_capf, s.y[0]))
                    return finish(s, out, ray, BHK_RAY_CAPTURED, ctl, G.r_cap);
                // Not proven in FP32: decide in FP64 (src/kerr.h:167-172 -- R near a turning point).
                if (no_radial_root_below(G.a, L.E[ray], L.L[ray], L.Q[ray], double(s.y[0]), p.eps))
                    return finish(s, out, ray, BHK_RAY_CAPTURED, ctl, G.r_cap);
                return kRescue;
            }
        }
        if constexpr (!F64) {
            // Pole reflection (kerr::normalizeAngles) in the hemisphere representation, carrying the
            // FSAL derivative: under theta -> -theta Theta'(theta) changes sign.
            if (s.y[1] < T(0)) {  // over the pole of this hemisphere
                s.y[1] = -s.y[1];
                s.y[2] += T(kPi);
                s.y[4] = -s.y[4];
                s.k[6][4] = -s.k[6][4];
            }
            if (s.y[1] > T(0.5 * kPi)) {  // across the equator: the other hemisphere's representation
                s.y[1] = T(kPi) - s.y[1];
                s.y[4] = -s.y[4];
                s.k[6][4] = -s.k[6][4];
                s.south = !s.south;
            }
            if (s.acc >= p.max_steps) return finish(s, out, ray, BHK_RAY_UNFINISHED, ctl);
        }
    }
    // Pole reflection (kerr::normalizeAngles) and constraint re-projection (kerr::enforceConstraints),
    // carrying the FSAL derivative: under theta -> -theta (or 2 pi - theta) Theta'(theta) changes sign.
    if constexpr (F64) {
        St st{0.0, s.y[0], s.y[1], s.y[2], s.y[3], s.y[4]};
        if (normalize_angles(st)) s.k[6][4] = -s.k[6][4];
        const Cons cc{s.c.E, s.c.L, s.c.Q, 0.0};
        enforce_constraints(s.c.a, cc, st);
        s.y[1] = st.theta; s.y[2] = st.phi; s.y[3] = st.vr; s.y[4] = st.vtheta;
    } else {
        // Every step, from the FSAL stage's potentials: keeps the FP32 rounding of vr ~ r^2 made
        // far out from becoming an O(1) error near the hole.
        if (pj.R > pj.Rz) s.y[3] = copysignf(sqrt_approx(pj.R), s.y[3]);
        if (pj.Th > pj.Thz) s.y[4] = copysignf(sqrt_approx(pj.Th), s.y[4]);
        if (reproject) {
            // Optional FP64 radial re-projection: R(r) = P^2 - Delta K evaluated in FP64.
            const double a = geom[L.geom_id[ray]].a, E = L.E[ray], Lz = L.L[ray], Q = L.Q[ray];
            const double r = double(s.y[0]);
            const double delta = r * r - 2.0 * r + a * a;
            const double P = E * (r * r + a * a) - a * Lz;
            const double x = Lz - a * E;
            const double K = x * x + Q;
            const double R = P * P - delta * K;
            if (R > 0.05 * (P * P + fabs(delta) * K)) s.y[3] = T(copysign(sqrt(R), double(s.y[3])));
        }
    }
#pragma unroll
    for (int i = 0; i < 5; ++i) s.k[0][i] = s.k[6][i];
    s.k[0][0] = s.y[3];
    s.k[0][1] = s.y[4];
    if constexpr (F64) s.kt[0] = s.kt[6];
    T fac;
    if constexpr (F64) fac = err > 0.0 ? 0.9 * pow(err, -0.2) : 5.0;
    else fac = e2 > 0.0f ? 0.9f * exp2f(-0.1f * __log2f(e2)) : 5.0f;
    fac = fmin(fmax(fac, T(0.2)), s.last_rej ? T(1) : T(5));
    s.h = h * fac;
    if constexpr (!F64) {
        // Outgoing, r(tau) ~ 1 / (E (tau_inf - tau)) runs into a pole at finite Mino time: the step
        // the tolerance allows shrinks geometrically and the error-per-step controller, which only
        // looks back, overshoots into a rejection every other step. Cap the step at a fixed fraction
        // of the Mino time left to the pole, ~ r / |vr|.
        // Outgoing: |r| grew over the step just taken (past |a| = 1 the r < 0 region has the same
        // pole); not within 2 M of r = 0, where the cap would vanish.
        if (p.pole_frac > 0.0f && falling == (s.y[0] < 0.0f) && fabsf(s.y[0]) > 2.0f) {
            const float cap = p.pole_frac * fabsf(s.y[0]) * rcp_approx(fabsf(s.y[3]));
            s.h = copysignf(fminf(fabsf(s.h), cap), s.h);
        }
    }
    s.last_rej = false;
    if constexpr (F64) {
        if (s.acc >= p.max_steps) return finish(s, out, ray, BHK_RAY_UNFINISHED, ctl);
    }
    return kContinue;
}

__device__ __forceinline__ void push_rescue(Rescue* rescue, unsigned cap, Control* ctl, long long ray, const double y[5],
                                            double h, double r_min, int acc, int rej, int from_launch,
                                            const Outputs& out) {
    const unsigned idx = atomicAdd(&ctl->rescue_count, 1u);
    atomicAdd(&ctl->stats[3], 1ull);
    if (idx < cap) {
        Rescue r;
        for (int i = 0; i < 5; ++i) r.y[i] = y[i];
        r.h = h; r.r_min = r_min; r.ray = ray; r.accepted = acc; r.rejected = rej; r.from_launch = from_launch;
        r.pad = 0;
        rescue[idx] = r;
    } else {
        write_out(out, ray, BHK_RAY_UNFINISHED, nan_d(), nan_d(), nan_d(), nan_d(), nan_d(), acc, rej);
        atomicAdd(&ctl->stats[2], 1ull);
    }
}

// kMinBlocks > 0 caps registers through __launch_bounds__(128, kMinBlocks) (blocks of <= 128 threads):
// 5 -> <= 102 registers (20 warps/SM), 6 -> <= 85 (24 warps/SM); 0 leaves the compiler free (blocks
// of <= 256 threads).
template <typename T, int kMinBlocks, bool kTP = false>
__global__ void __launch_bounds__(kMinBlocks > 0 ? 128 : 256, kMinBlocks > 0 ? kMinBlocks : 1)
trace_kernel(LaunchSoA L, const RayGeom* __restrict__ geom, const int32_t* __restrict__ order,
             Outputs out, Rescue* rescue, unsigned rescue_cap, TraceParams p, Control* ctl,
             const FrameDev* __restrict__ frames, int nframes) {
    const int lane = threadIdx.x & 31;
    const long long n = ctl->n_rays;
    Lane<T> s;
    // A batch holds < 2^31 rays (the API refuses more), so queue positions and ray indices fit 32 bits.
    int ray = -1;
    bool exhausted = false;
    int pool_pos = 0, pool_end = 0;  // this warp's chunk of the queue
    // Per-lane step counts, flushed to the 64-bit totals before they can wrap (a ray adds < 2^31).
    unsigned n_acc = 0, n_rej = 0, n_tp = 0;
    for (;;) {
        // A warp traces its rays in batches of 32 queue-adjacent rays -- neighbouring pixels, or rays
        // of one cost bucket -- and takes the next batch only when every lane's ray has ended. Rays
        // that start together stay alike (similar step sizes, events and branches) for their whole
        // path; refilling lanes one by one mixes rays at different stages within the warp, and the
        // divergence that follows costs more than the lanes that wait for their batch's last ray.
        // A lane traces while its ray has not ended (FP64 lanes drop the ray as it ends).
        const bool active = ray >= 0 && s.pend < 0;
        if (!__any_sync(kFull, active)) {
            // The batch is over: its FP32 results are written together, then the next one is taken.
            if constexpr (sizeof(T) == 4) {
                if (ray >= 0) flush_f32(s, out, ray, ctl, geom, L);
            }
            ray = -1;
            if (exhausted) break;
            if (pool_pos >= pool_end) {
                unsigned long long base = 0;
                if (lane == 0) base = atomicAdd(&ctl->queue, static_cast<unsigned long long>(p.chunk));
                base = __shfl_sync(kFull, base, 0);
                if (static_cast<long long>(base) >= n) {
                    exhausted = true;
                    break;
                }
                pool_pos = static_cast<int>(base);
                pool_end = static_cast<int>(base + p.chunk < static_cast<unsigned long long>(n) ? base + p.chunk : n);
            }
            const int q = pool_pos + lane;
            if (q < pool_end) {
                // Frames: queue position -> pixel by 8 x 4 tiles (the frame is the same for both).
                int fi = 0, prow = 0, pcol = 0;
                if (frames) {
                    fi = frame_of(frames, nframes, q);
                    const FrameDev& f = frames[fi];
                    tile_pixel(f.d.width, f.d.height, static_cast<int>(q - f.offset), &prow, &pcol);
                    ray = static_cast<int>(f.offset) + prow * f.d.width + pcol;
                } else {
                    ray = order ? order[q] : q;
                }
                // Frames: the launch is made here, by the whole warp at once, so that its FP64
                // arithmetic overlaps other warps' FP32 integration instead of taking a kernel of its
                // own; only the FP64 record (for the FP64 continuation and the RayReport constants)
                // is stored.
                if constexpr (sizeof(T) == 4) {
                    if (frames) {
                        const Launched x = photon_at(frames[fi], fi, prow, pcol);
                        L.E[ray] = x.E; L.L[ray] = x.L; L.Q[ray] = x.Q; L.vr[ray] = x.vr; L.vth[ray] = x.vth;
                        L.geom_id[ray] = x.gid;
                        const RayGeom& G = geom[x.gid];
                        const double xk = x.L - G.a * x.E;
                        lane_begin_f32(s, G, make_float4(float(x.E), float(x.L), float(x.Q), float(xk * xk + x.Q)),
                                       make_float2(float(x.vr), float(x.vth)), float4{}, float2{}, false, p);
                    } else {
                        const RayGeom& G = geom[L.geom_id[ray]];
                        const float4 k = L.kf ? L.kf[ray] : float4{};
                        const float2 kh = L.khf ? L.khf[ray] : float2{};
                        lane_begin_f32(s, G, L.cf[ray], L.vf[ray], k, kh, L.kf != nullptr, p);
                    }
                } else {
                    if (frames) launch_pixel(frames, geom, nframes, ray, ray, L, p);
                    lane_begin_launch(s, geom[L.geom_id[ray]], L, ray, p);
                }
                const RayGeom& G = geom[L.geom_id[ray]];
                if (G.dead) {  // seen from inside the horizon: the hole, with no step taken
                    finish(s, out, ray, BHK_RAY_CAPTURED, ctl, G.r_cap);
                    if constexpr (sizeof(T) == 8) ray = -1;
                }
            }
            pool_pos = pool_pos + 32 < pool_end ? pool_pos + 32 : pool_end;
            continue;
        }
        if (active) {
            // The optional FP64 re-projection on every reproject_every-th attempt of the ray.
            const bool reproject = p.reproject_every > 0 && (s.acc + s.rej + 1) % p.reproject_every == 0;
            const int r = attempt<T, kTP>(s, p, ray, out, reproject, ctl, L, geom, &n_tp);
            if (r != kContinue) {
                n_acc += static_cast<unsigned>(s.acc);
                n_rej += static_cast<unsigned>(s.rej);
                if ((n_acc | n_rej) >= (1u << 30)) {
                    atomicAdd(&ctl->stats[0], static_cast<unsigned long long>(n_acc));
                    atomicAdd(&ctl->stats[1], static_cast<unsigned long long>(n_rej));
                    n_acc = 0;
                    n_rej = 0;
                }
                if (r == kRescue || r == kRestart) {
                    double y[5];
                    const bool restart = r == kRestart;
                    if (restart) {
                        const RayGeom& g = geom[L.geom_id[ray]];
                        y[0] = g.r0; y[1] = g.th0; y[2] = g.ph0; y[3] = L.vr[ray]; y[4] = L.vth[ray];
                    } else {
                        for (int i = 0; i < 5; ++i) y[i] = double(s.y[i]);
                        if (s.south) {
                            y[1] = kPi - y[1];
                            y[4] = -y[4];
                        }
                    }
                    push_rescue(rescue, rescue_cap, ctl, ray, y, restart ? 0.0 : double(s.h),
                                restart ? y[0] : fmin(double(s.rmin), y[0]), restart ? 0 : s.acc,
                                restart ? 0 : s.rej, restart ? 1 : 0, out);
                    ray = -1;
                } else if constexpr (sizeof(T) == 8) {
                    ray = -1;  // written as it ended
                }
            }
        }
    }
    // Step statistics: one atomic per warp.
    unsigned long long t_acc = n_acc, t_rej = n_rej;
    for (int o = 16; o > 0; o >>= 1) {
        t_acc += __shfl_down_sync(kFull, t_acc, o);
        t_rej += __shfl_down_sync(kFull, t_rej, o);
    }
    if (lane == 0) {
        atomicAdd(&ctl->stats[0], t_acc);
        atomicAdd(&ctl->stats[1], t_rej);
    }
    if constexpr (kTP) {
        if (n_tp) atomicAdd(&ctl->stats[4], static_cast<unsigned long long>(n_tp));
    }
}

// FP64 continuation of the rays the FP32 kernel handed over; one thread per record.
__global__ void rescue_kernel(LaunchSoA L, const RayGeom* __restrict__ geom, Outputs out, const Rescue* rescue,
                              unsigned cap, TraceParams p, Control* ctl) {
    const unsigned count = ctl->rescue_count < cap ? ctl->rescue_count : cap;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const Rescue r = rescue[i];
        const RayGeom& g = geom[L.geom_id[r.ray]];
        Lane<double> s;
        if (r.from_launch) {
            lane_begin_launch(s, g, L, r.ray, p);
        } else {
            St st{0.0, r.y[0], r.y[1], r.y[2], r.y[3], r.y[4]};
            normalize_angles(st);
            const Cons cc{L.E[r.ray], L.L[r.ray], L.Q[r.ray], 0.0};
            enforce_constraints(g.a, cc, st);
            s.c.set(g.a, cc.E, cc.L, cc.Q);
            s.south = false;
            s.y[0] = st.r; s.y[1] = st.theta; s.y[2] = st.phi; s.y[3] = st.vr; s.y[4] = st.vtheta;
            lane_radii(s, g);
            rhs(s.c, s.y, s.k[0]);
            s.h = r.h;
            s.last_rej = false;
        }
        s.acc = r.accepted;
        s.rej = r.rejected;
        s.rmin = r.r_min;
        s.track = false;  // the FP32 part kept no time or swept angle
        s.t = 0.0;
        s.swept = 0.0;
        s.pend = -1;
        int res = kContinue;
        while (res == kContinue) res = attempt<double>(s, p, r.ray, out, false, ctl, L, geom);
        atomicAdd(&ctl->stats[0], static_cast<unsigned long long>(s.acc - r.accepted));
        atomicAdd(&ctl->stats[1], static_cast<unsigned long long>(s.rej - r.rejected));
    }
}

// trajectory::traceRay's energy, gCamera, b, q (src/trajectory.cpp:219-224) from the FP64 launch.
__global__ void constants_out_kernel(LaunchSoA L, Outputs out, const Control* __restrict__ ctl) {
    const long long n = ctl->n_rays;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const double E = L.E[i];
        const double invE = fabs(E) > 1e-12 ? 1.0 / E : 0.0;
        if (out.energy) out.energy[i] = E;
        if (out.g_camera) out.g_camera[i] = invE;
        if (out.b) out.b[i] = L.L[i] * invE;
        if (out.q) out.q[i] = L.Q[i] * invE * invE;
    }
}

// Analytic critical curve seen by a ZAMO pinhole (one thread per spherical-orbit sample).
__global__ void critical_curve_kernel(double a, double r_obs, double th, int samples, double* alpha, double* beta,
                                      int* valid) {
    const int n = (samples > 16 ? samples : 16) * 8;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k > n) return;
    double al, be;
    valid[k] = critical_point(a, r_obs, th, static_cast<double>(k) / n, &al, &be) ? 1 : 0;
    alpha[k] = al;
    beta[k] = be;
}

}  // namespace

// ------------------------------------------------------------------------------ launchers ----

void launch_frame_setup(FrameDev* frames, RayGeom* geom, int nframes, const TraceParams& p, Control* ctl,
                        cudaStream_t s) {
    frame_setup_kernel<<<1, 128, 0, s>>>(frames, geom, nframes, p, ctl);
}

long long setup_frames_host(FrameDev* frames, RayGeom* geom, int nframes, const TraceParams& p) {
    long long off = 0;
    for (int f = 0; f < nframes; ++f) {
        frames[f].offset = off;
        off += static_cast<long long>(frames[f].d.width) * frames[f].d.height;
        setup_frame(frames[f], geom[f], p);
    }
    return off;
}

void launch_rays_frames(const FrameDev* frames, const RayGeom* geom, int nframes, LaunchSoA L, const TraceParams& p,
                        const Control* ctl, int grid, cudaStream_t s) {
    launch_frames_kernel<<<grid, 128, 0, s>>>(frames, geom, nframes, L, p, ctl);
}

void launch_rays_framed(const double* a, const double* r, const double* th, const double* ph, const bhk_frame* frames,
                        const double* look, double r_in, double r_out, RayGeom* geom, LaunchSoA L, const TraceParams& p,
                        const Control* ctl, int grid, cudaStream_t s) {
    launch_framed_kernel<<<grid, 128, 0, s>>>(a, r, th, ph, frames, look, r_in, r_out, geom, L, p, ctl);
}

void launch_rays_list(const FrameDev* frames, const RayGeom* geom, int nframes, const int32_t* list, LaunchSoA L,
                      const TraceParams& p, const Control* ctl, int grid, cudaStream_t s) {
    launch_list_kernel<<<grid, 128, 0, s>>>(frames, geom, nframes, list, L, p, ctl);
}

void launch_rays_explicit(const double* a, const double* r_obs, const double* th_obs, const double* alpha,
                          const double* beta, double r_in, double r_out, RayGeom* geom, LaunchSoA L,
                          const TraceParams& p, const Control* ctl, int grid, cudaStream_t s) {
    launch_explicit_kernel<<<grid, 128, 0, s>>>(a, r_obs, th_obs, alpha, beta, r_in, r_out, geom, L, p, ctl);
}

void launch_sort(LaunchSoA L, SortScratch S, const TraceParams& p, const Control* ctl, int grid, cudaStream_t s) {
    hist_kernel<<<grid, 256, 0, s>>>(L, S, p, ctl);
    scan_kernel<<<1, 32, 0, s>>>(S, p);
    scatter_kernel<<<grid, 256, 0, s>>>(L, S, p, ctl);
}

namespace {
using TraceFn = void (*)(LaunchSoA, const RayGeom*, const int32_t*, Outputs, Rescue*, unsigned, TraceParams, Control*,
                         const FrameDev*, int);

// Variant by precision and register cap (see trace_kernel); FP64 attempts near turning points have
// their own variant at the <= 102-register cap.
TraceFn trace_variant(bool fp64, int regcap, bool tp = false) {
    if (fp64) return trace_kernel<double, 0>;
    if (tp) return trace_kernel<float, 5, true>;
    if (regcap == 1) return trace_kernel<float, 5>;
    if (regcap == 2) return trace_kernel<float, 6>;
    return trace_kernel<float, 0>;
}
}  // namespace

void launch_trace(bool fp64, int regcap, LaunchSoA L, const RayGeom* geom, const int32_t* order, Outputs out,
                  Rescue* rescue, unsigned rescue_cap, const TraceParams& p, Control* ctl, int block, int grid,
                  cudaStream_t s, const FrameDev* frames, int nframes) {
    trace_variant(fp64, regcap, !fp64 && p.fp64_turning)<<<grid, block, 0, s>>>(L, geom, order, out, rescue,
                                                                                  rescue_cap, p, ctl, frames, nframes);
}

void launch_constants_out(LaunchSoA L, Outputs out, const Control* ctl, int grid, cudaStream_t s) {
    if (out.energy || out.g_camera || out.b || out.q) constants_out_kernel<<<grid, 128, 0, s>>>(L, out, ctl);
}

void launch_rescue(LaunchSoA L, const RayGeom* geom, Outputs out, Rescue* rescue, unsigned rescue_cap,
                   const TraceParams& p, Control* ctl, int grid, cudaStream_t s) {
    rescue_kernel<<<grid, 64, 0, s>>>(L, geom, out, rescue, rescue_cap, p, ctl);
}

int trace_blocks_per_sm(bool fp64, int regcap, int block) {
    if (block > 256 || (regcap > 0 && (fp64 || block > 128))) return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, trace_variant(fp64, regcap), block, 0) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

void launch_critical_curve(double a, double r_obs, double theta_obs, int samples, double* alpha, double* beta,
                           int* valid, cudaStream_t s) {
    const int n = (samples > 16 ? samples : 16) * 8 + 1;
    critical_curve_kernel<<<(n + 127) / 128, 128, 0, s>>>(a, r_obs, theta_obs, samples, alpha, beta, valid);
}

}  // namespace bhk
