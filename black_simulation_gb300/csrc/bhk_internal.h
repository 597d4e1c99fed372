// bhk_internal.h -- device-memory layouts and kernel launchers shared by the tracer and the C ABI.
#pragma once

#include <cstdint>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "../../include/bhk.h"

namespace bhk {

// Per-camera geometry the tracer needs for every ray of that camera (FP64, computed on device),
// with FP32 copies for the FP32 tracer (which then issues no FP64 conversions per ray).
struct RayGeom {
    double a, r0, th0, ph0;       // camera position = launch point
    double rp, r_cap, r_esc;      // horizon, capture and escape radii
    double r_in, r_out, zone_top; // disk, and r_+ + width of the analytic capture zone
    float af, r0f, th0f, ph0f, r_capf, r_escf, r_inf, r_outf, zone_topf, rpf;
    int32_t south0;               // camera below the equator: th0f holds pi - theta_obs
    int32_t dead;                 // per-ray geometry only: a camera inside the horizon sees the hole
                                  // (trajectory::traceRay's rule, src/trajectory.cpp:236-244)
    int32_t naked;                // |a| > 1: no horizon (r_cap, zone_top at -1e30); the ring and the
                                  // sky beyond it end rays instead (shaders/trace.frag:1772-1787)
    int32_t pad;
};

// Frame descriptor after set-up: pixel mapping, frame tetrad, ray offset, and the per-camera
// pieces of kerr::photonFromFrame (src/kerr.cpp:458-483) hoisted out of the per-ray launch.
struct FrameDev {
    bhk_frame_desc d;
    int64_t offset;               // first global ray index of this frame
    double e[4][4];               // ZAMO frame at the camera
    double el[4][4];              // the same vectors lowered with the camera's metric, g e_k
    double sigma, cs2, inv_sn2, a2;  // Sigma, cos^2, 1/max(sin^2, 1e-18), a^2 at the camera
    double inv_r, px, py;         // 1/r_obs and the pixel pitch in alpha and beta
};

// Launch record of one ray, structure of arrays, written by the FP64 launch kernel: the FP64
// constants, and their FP32 roundings for the FP32 tracer -- (E, L, Q, K = (L - aE)^2 + Q) and
// (vr, vtheta) -- so that it loads ready operands.
struct LaunchSoA {
    double *E, *L, *Q, *vr, *vth;
    int32_t* geom_id;             // index into the RayGeom table
    uint16_t* key;                // cost bucket for the pre-sort
    float4* cf;
    float2* vf;
    // FP32 runs only (nullptr otherwise): the FP32 tracer's first step, prepared by the launch kernel
    // so that a lane picking up a ray does no arithmetic on its own -- the right-hand side at the
    // launch point (k[0..3] in kf, k[4] and the first step h in khf).
    float4* kf;
    float2* khf;
};

// Small control block reset at the start of every batch.
struct Control {
    unsigned long long queue;     // next position in the ray queue
    unsigned long long stats[5];  // accepted steps, rejected steps, unfinished rays, rescued rays,
                                  // FP64 attempts near turning points
    long long n_rays;             // total rays of the batch (device-resident: graph friendly)
    unsigned int rescue_count;
    unsigned int pad;
};

constexpr int kMaxBuckets = 1024;

struct SortScratch {
    unsigned int* hist;           // kMaxBuckets counters
    unsigned int* offs;           // kMaxBuckets running offsets
    int32_t* order;               // queue position -> ray index
};

// A ray the FP32 tracer hands to FP64 (capture zone inconclusive, or non-finite state).
struct Rescue {
    double y[5];
    double h;
    double r_min;                 // closest approach so far
    int64_t ray;
    int32_t accepted, rejected;
    int32_t from_launch, pad;
};

struct TraceParams {
    double rtol, eps, r_escape;
    int32_t max_steps, reproject_every, chunk, buckets;
    double tol0;                  // photonStepSize tolerance of the first step
    float rtol_f, tol0_f;         // the same for the FP32 path (no conversions in the loop)
    float pole_frac;              // FP32: outgoing steps capped at pole_frac * r / |vr| (0 = no cap)
    int32_t fp64_turning;         // FP32: attempts near turning points in FP64 (bhk_trace_opts.fp64_turning)
    int32_t pad;
};

struct Outputs {
    uint8_t* outcome;
    double *r_disk, *phi_disk, *g, *theta_inf, *phi_inf;
    int32_t* steps;
    int32_t* rejected;
    double *energy, *g_camera, *b, *q, *r_min, *delay, *turns;  // optional (NULL: not written)
};

// ---- launchers (bhk_trace.cu) ----
void launch_frame_setup(FrameDev* frames, RayGeom* geom, int nframes, const TraceParams& p, Control* ctl,
                        cudaStream_t s);
// The same set-up on the host (the frame table's offsets, tetrads and geometries); returns the rays.
long long setup_frames_host(FrameDev* frames, RayGeom* geom, int nframes, const TraceParams& p);
void launch_rays_frames(const FrameDev* frames, const RayGeom* geom, int nframes, LaunchSoA L, const TraceParams& p,
                        const Control* ctl, int grid, cudaStream_t s);
void launch_rays_list(const FrameDev* frames, const RayGeom* geom, int nframes, const int32_t* list, LaunchSoA L,
                      const TraceParams& p,
                      const Control* ctl, int grid, cudaStream_t s);
void launch_rays_explicit(const double* a, const double* r_obs, const double* th_obs, const double* alpha,
                          const double* beta, double r_in, double r_out, RayGeom* geom, LaunchSoA L,
                          const TraceParams& p, const Control* ctl, int grid, cudaStream_t s);
// Per-ray cameras with arbitrary frames (moving, or inside the horizon): kerr::photonFromFrame.
void launch_rays_framed(const double* a, const double* r, const double* th, const double* ph, const bhk_frame* frames,
                        const double* look, double r_in, double r_out, RayGeom* geom, LaunchSoA L, const TraceParams& p,
                        const Control* ctl, int grid, cudaStream_t s);
void launch_sort(LaunchSoA L, SortScratch S, const TraceParams& p, const Control* ctl, int grid, cudaStream_t s);
// With frames (frame batches traced in queue order without the cost sort), the trace kernel makes
// each ray's launch record itself when it takes the ray; otherwise the records come from a launch
// kernel run before it.
void launch_trace(bool fp64, int regcap, LaunchSoA L, const RayGeom* geom, const int32_t* order, Outputs out,
                  Rescue* rescue, unsigned rescue_cap, const TraceParams& p, Control* ctl, int block, int grid,
                  cudaStream_t s, const FrameDev* frames = nullptr, int nframes = 0);
// energy, g_camera, b, q of every ray from its FP64 launch constants (if any is requested).
void launch_constants_out(LaunchSoA L, Outputs out, const Control* ctl, int grid, cudaStream_t s);
// grid: one block of 64 threads per SM is plenty (rescued rays are rare).
void launch_rescue(LaunchSoA L, const RayGeom* geom, Outputs out, Rescue* rescue, unsigned rescue_cap,
                   const TraceParams& p, Control* ctl, int grid, cudaStream_t s);
int trace_blocks_per_sm(bool fp64, int regcap, int block);  // 0 when the pair is not allowed
void launch_critical_curve(double a, double r_obs, double theta_obs, int samples, double* alpha, double* beta,
                           int* valid, cudaStream_t s);

// Sets the text bhk_last_error() returns on this thread (bhk_api.cu).
void set_last_error(const std::string& msg);

// The frame checks of bhk_trace_frames (bhk_api.cu): sizes, spin (|a| != 1; naked singularities
// allowed), camera outside the horizon, theta_obs in (0, pi), r_disk_out >= 0, < 2^31 rays. Sets the
// last error and returns BHK_EINVAL on the first bad frame; *total receives the ray count.
bhk_status validate_frames(const bhk_frame_desc* f, int32_t nframes, int64_t* total);

// ---- context internals for the other translation units (bhk_api.cu) ----
// Traces pixels list[0..n) (device memory, global pixel indices of the frames) into `out` (compact:
// entry i is pixel list[i]), or into context-owned device buffers when out is null; *used (if given)
// receives the buffers written. The caller holds context_mutex(c) and has selected the device.
bhk_status trace_pixel_list(bhk_context* c, const bhk_frame_desc* frames, int32_t nframes, const int32_t* list,
                            int64_t n, const bhk_trace_opts* opts, const bhk_rays_out* out, bhk_rays_out* used,
                            cudaStream_t s);
std::mutex& context_mutex(bhk_context* c);
cudaStream_t context_stream(bhk_context* c, void* stream);  // stream, or the context's own when null
int context_device(bhk_context* c);

// ---- per-step mirrors (bhk_steps.cu) ----
cudaError_t steps_derivatives(double a, const bhk_constants* c, const bhk_state* s, bhk_derivatives_t* d, int64_t n,
                              cudaStream_t st);
cudaError_t steps_step_mino(double a, const bhk_constants* c, bhk_state* s, const double* h, int64_t n,
                            cudaStream_t st);
cudaError_t steps_photon_step_size(double a, const bhk_constants* c, const bhk_state* s, double tol, double* h,
                                   int64_t n, cudaStream_t st);
cudaError_t steps_enforce_constraints(double a, const bhk_constants* c, bhk_state* s, int64_t n, cudaStream_t st);
cudaError_t steps_normalize_angles(bhk_state* s, int64_t n, cudaStream_t st);
cudaError_t steps_potentials(double a, const bhk_constants* c, const bhk_state* s, double* R, double* Th, int64_t n,
                             cudaStream_t st);
cudaError_t steps_observer_frame(double a, const double* r, const double* th, const double* u, bhk_frame* f, int64_t n,
                                 cudaStream_t st);
cudaError_t steps_photon_from_frame(double a, double r, double th, double ph, const bhk_frame* f, const double* look,
                                    bhk_constants* c, bhk_state* s, int64_t n, cudaStream_t st);
cudaError_t steps_launch_from_zamo(double a, double r, double th, double ph, const double* v, double mu,
                                   bhk_constants* c, bhk_state* s, int64_t n, cudaStream_t st);
cudaError_t steps_predict(double a, const bhk_constants* c, const bhk_state* s, int64_t n, double max_time,
                          double min_spacing, int32_t max_points, double surface, double escape_radius,
                          bhk_state* s_out, const bhk_path_out& out, cudaStream_t st);
cudaError_t steps_cartesian_velocity(double a, const bhk_constants* c, const bhk_state* s, double* out, int64_t n,
                                     cudaStream_t st);

}  // namespace bhk
