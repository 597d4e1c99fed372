/*
 * bhk.h -- C ABI of libbhk, the GB300 (sm_103a) Kerr null-geodesic batch tracer.
 *
 * Drop-in for the photon path of Black_simulation: the kerr:: geodesic primitives
 * (src/kerr.h:101-185) and the ray-level drivers built on them, trajectory::traceRay
 * (src/trajectory.h:118-119) and eht::render / eht::traceRay (src/eht.h:130-140).
 *
 * Conventions
 *  - Units G = c = M = 1; ingoing Kerr-Schild (t, r, theta, phi); Mino time.
 *  - Every function returns a bhk_status. Nothing computes on the CPU: the per-step mirrors run
 *    the same FP64 device code as the tracer, batched over n items of device memory.
 *  - Pointers documented "device" must be device (or managed) memory; "host" must be host memory.
 *  - `stream` is a cudaStream_t passed as void* (NULL = the context's own stream). Calls are
 *    asynchronous on that stream unless documented otherwise.
 *  - A bhk_context is thread-safe: concurrent calls on one context are serialised by its lock.
 *    Separate contexts are independent.
 *  - No CPU fallback: without a CUDA device every call returns BHK_ECUDA.
 */
#ifndef BHK_H
#define BHK_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    BHK_OK = 0,
    BHK_EINVAL = 1,       /* bad argument (null pointer, size, range) */
    BHK_ECUDA = 2,        /* CUDA error; bhk_last_error() has the text */
    BHK_EUNFINISHED = 3,  /* traced, but some rays hit the step cap (outcome BHK_RAY_UNFINISHED) */
    BHK_ENOMEM = 4        /* device allocation failed */
} bhk_status;

/* Ray outcomes (trajectory::RayEnd, src/trajectory.h:85, restricted to a bare hole + thin disk).
 * Past |a| = 1 (a naked singularity, no horizon) nothing is captured; as the renderer has it
 * (shaders/trace.frag:1768-1787) a ray may instead strike the ring singularity (Sigma =
 * r^2 + a^2 cos^2 theta < 4e-4: BHK_RAY_RING) or pass through the ring's disk to the r < 0 region
 * and leave to that region's sky below r = -max(r_escape, 1.5 r_obs) (BHK_RAY_ESCAPED_BEYOND, with
 * theta_inf, phi_inf like BHK_RAY_ESCAPED). */
enum { BHK_RAY_UNFINISHED = 0, BHK_RAY_CAPTURED = 1, BHK_RAY_DISK = 2, BHK_RAY_ESCAPED = 3,
       BHK_RAY_ESCAPED_BEYOND = 4, BHK_RAY_RING = 5 };

/* Layout-identical to kerr::Constants, kerr::State, kerr::Derivatives, kerr::Frame
 * (src/kerr.h:81-99, 143-145). */
typedef struct { double E, L, Q, mu; } bhk_constants;
typedef struct { double t, r, theta, phi, vr, vtheta; } bhk_state;
typedef struct { double dt, dr, dtheta, dphi, dvr, dvtheta; } bhk_derivatives_t;
typedef struct { double e[4][4]; } bhk_frame; /* e[k][mu]: e[0] the 4-velocity, e[1..3] the r, theta, phi axes */

/* ------------------------------------------------------------------ context ---------------- */

typedef struct bhk_context bhk_context;

bhk_status bhk_create(int device, bhk_context** out);
bhk_status bhk_destroy(bhk_context* ctx);
const char* bhk_last_error(void);          /* thread-local text of the last failure */
const char* bhk_version(void);

/* ------------------------------------------------- per-step mirrors (batched) ---------------- */
/* Each applies the kerr:: function of the same name to n independent items, in FP64, on the GPU.
 * Spin a is shared by the batch, as in the reference call shape. All arrays are device memory. */

/* kerr::derivatives (src/kerr.h:101; src/kerr.cpp:331-351). */
bhk_status bhk_derivatives(double a, const bhk_constants* c, const bhk_state* s, bhk_derivatives_t* d, int64_t n,
                           void* stream);
/* kerr::stepMino: one classical RK4 step of Mino-time size h[i] (src/kerr.h:165; src/kerr.cpp:502-519). */
bhk_status bhk_step_mino(double a, const bhk_constants* c, bhk_state* s, const double* h, int64_t n, void* stream);
/* kerr::photonStepSize (src/kerr.h:176; src/kerr.cpp:563-575). */
bhk_status bhk_photon_step_size(double a, const bhk_constants* c, const bhk_state* s, double tolerance, double* h,
                                int64_t n, void* stream);
/* kerr::enforceConstraints (src/kerr.h:173; src/kerr.cpp:521-542). */
bhk_status bhk_enforce_constraints(double a, const bhk_constants* c, bhk_state* s, int64_t n, void* stream);
/* kerr::normalizeAngles (src/kerr.h:185; src/kerr.cpp:595-604). */
bhk_status bhk_normalize_angles(bhk_state* s, int64_t n, void* stream);
/* kerr::radialPotential / polarPotential (src/kerr.h:103-104; src/kerr.cpp:353-363). */
bhk_status bhk_potentials(double a, const bhk_constants* c, const bhk_state* s, double* R, double* Theta, int64_t n,
                          void* stream);
/* kerr::observerFrame(a, r[i], theta[i], u[i]) (src/kerr.h:146; src/kerr.cpp:432-456). u: n x 4.
 * u == NULL uses each point's ZAMO 4-velocity, kerr::zamoFourVelocity (src/kerr.cpp:424-430). */
bhk_status bhk_observer_frame(double a, const double* r, const double* theta, const double* u, bhk_frame* f,
                              int64_t n, void* stream);
/* kerr::photonFromFrame for one camera and n look directions (look: n x 3, unit, on the frame's
 * r, theta, phi axes), including the kAxisSnap rewrite (src/kerr.h:153-154; src/kerr.cpp:458-483).
 * frame is a device pointer to one bhk_frame. */
bhk_status bhk_photon_from_frame(double a, double r, double theta, double phi, const bhk_frame* frame,
                                 const double* look, bhk_constants* c, bhk_state* s, int64_t n, void* stream);
/* kerr::launchFromZamo for n directions v (n x 3) from one point (src/kerr.h:124-125; src/kerr.cpp:365-407). */
bhk_status bhk_launch_from_zamo(double a, double r, double theta, double phi, const double* v, double mu,
                                bhk_constants* c, bhk_state* s, int64_t n, void* stream);
/* kerr::cartesianVelocity applied to each state with its own derivatives: out (n x 3) is the
 * Cartesian direction of motion, unnormalised (src/kerr.cpp:651-658). */
bhk_status bhk_cartesian_velocity(double a, const bhk_constants* c, const bhk_state* s, double* out, int64_t n,
                                  void* stream);

/* ------------------------------------------------------------- batch tracer ---------------- */

/* One camera frame: a ZAMO pinhole at (r_obs, theta_obs, phi_obs) around a hole of spin a.
 * Pixel (col, row), row-major from the top, looks along normalize(-1, -beta/r_obs, alpha/r_obs) on the
 * ZAMO's (r, theta, phi) axes, with alpha = alpha_lo + (col + 1/2)(alpha_hi - alpha_lo)/width and
 * beta = beta_hi - (row + 1/2)(beta_hi - beta_lo)/height (the image layout of eht::render,
 * src/eht.cpp:332-336; the launch is kerr::photonFromFrame, src/kerr.cpp:458-483). As r_obs grows,
 * (alpha, beta) become Bardeen's impact parameters (src/eht.cpp:263-264). */
typedef struct {
    double a, r_obs, theta_obs, phi_obs;
    int32_t width, height;
    double alpha_lo, alpha_hi, beta_lo, beta_hi;
    double r_disk_in;   /* <= 0: the prograde ISCO, kerr::iscoRadius(a, true) */
    double r_disk_out;  /* 0: no disk (a shadow-only image, as eht::render's) */
} bhk_frame_desc;

enum { BHK_PREC_FP64 = 0, BHK_PREC_MIXED = 1 };

typedef struct {
    int32_t precision;      /* BHK_PREC_FP64 (parity mode) or BHK_PREC_MIXED (FP32 integration) */
    double rtol;            /* Dormand-Prince relative (= absolute) tolerance; 0 -> 1e-10 FP64, 1e-6 mixed */
    int32_t max_steps;      /* accepted-step cap per ray; 0 -> 20000 */
    double r_escape;        /* escaped once r > max(r_escape, 1.5 r_obs) while rising; 0 -> 1000 */
    double capture_eps;     /* captured once r < r_+(1 + capture_eps) while falling; 0 -> 1e-6 */
    int32_t reproject_every;/* mixed: besides the FP32 re-projection every step, an FP64 radial one on every
                               N-th step attempt of a ray; 0 = off */
    int32_t block;          /* threads per block of the tracer; 0 -> autotuned or 128 */
    int32_t chunk;          /* rays a warp takes from the queue at a time, traced in batches of 32 (one
                               per lane; the next batch starts when all 32 have ended); rounded up to a
                               multiple of 32; 0 -> autotuned or 32 */
    int32_t sort_buckets;   /* rays pre-sorted into this many cost buckets; 0 -> autotuned or 1; 1 = none
                               (frames are then taken by 8 x 4 pixel tiles and launched in the kernel) */
    int32_t use_graph;      /* 1: replay the whole batch as one captured CUDA graph */
    int32_t reg_budget;     /* mixed tracer variant: 0 autotuned (else 1), 1: <= 102 registers per
                               thread (20 warps/SM, blocks <= 128), 2: <= 85 (24 warps/SM), 3: uncapped */
    double pole_step_frac;  /* mixed: outgoing steps capped at this fraction of the Mino time left before
                               r runs off to infinity (~ r/|vr|); 0 -> 0.1 (rtol/1e-6)^(1/5), < 0 off */
    int32_t fp64_turning;   /* mixed, 1: a step that starts within ~0.05 M of a radial turning point (vr^2 <
                               0.1 |R'/2|) or ~0.05 rad of a polar one (vtheta^2 < 0.1 |Theta'/2|) is taken in
                               FP64 (its stages, error estimate and constraint potentials), from the FP64 launch
                               constants; its own compiled variant (<= 102 registers). 0: off (the default) */
    int32_t pad;
} bhk_trace_opts;

/* Per-ray outputs, structure of arrays, n entries each (device memory unless stated). Any pointer
 * may be NULL to skip that field. Undefined fields (r_disk of an escaped ray, ...) are NaN. */
typedef struct {
    uint8_t* outcome;    /* BHK_RAY_* */
    double* r_disk;      /* disk-crossing radius (trajectory RayReport::rEnd for RayEnd::Disk) */
    double* phi_disk;    /* Kerr-Schild azimuth of the crossing, wrapped to [0, 2 pi) */
    double* g;           /* observed / emitted frequency, gas on prograde circular orbits (RayReport::g) */
    double* theta_inf;   /* escape direction, backward tangent at r_escape: acos(d_z) */
    double* phi_inf;     /*                                                 atan2(d_y, d_x) */
    int32_t* steps;      /* accepted integration steps */
    int32_t* rejected;   /* rejected integration steps */
    /* The rest of trajectory::RayReport (src/trajectory.h:95-113); NULL pointers are not written. */
    double* energy;      /* E for unit energy at the camera (RayReport::energy) */
    double* g_camera;    /* 1 / E (RayReport::gCamera) */
    double* b;           /* L / E (RayReport::b) */
    double* q;           /* Q / E^2 (RayReport::q) */
    double* r_min;       /* closest approach (RayReport::rMin): refined at the radial turning point by the
                            dense output; r_+(1 + eps) for captured rays */
    double* delay;       /* Kerr-Schild time the light spent travelling (RayReport::delay); FP64 mode only
                            (NaN in the mixed mode) */
    double* turns;       /* angle swept by the position around the hole / 2 pi (RayReport::turns), as the
                            reference sums it over the steps; FP64 mode only (NaN in the mixed mode) */
} bhk_rays_out;

/* Statistics of the last trace call on a context (filled at the end of that call's stream work). */
typedef struct {
    int64_t rays, accepted_steps, rejected_steps, rescued, unfinished;
    int32_t block, chunk, sort_buckets, grid, reg_budget, pad;
    double kernel_ms;    /* CUDA events on the launching stream: tracer + rescue kernels, or the
                            whole batch when it ran as a CUDA graph */
    int64_t fp64_turning_steps;  /* step attempts taken in FP64 near turning points (fp64_turning) */
} bhk_trace_stats;

/* Traces every pixel of nframes frames (host descriptors) in one persistent launch. Ray i of frame f
 * is written at offset (sum of earlier frames' pixels) + i. Outputs are device memory. Returns
 * BHK_EUNFINISHED if any ray hit the step cap (after synchronising the stream), else BHK_OK. */
bhk_status bhk_trace_frames(bhk_context* ctx, const bhk_frame_desc* frames, int32_t nframes,
                            const bhk_trace_opts* opts, const bhk_rays_out* out, void* stream);
/* The same with HOST output buffers, synchronous: the eht::render-style call (src/eht.cpp:321-347),
 * frames in, images out, in host memory. Page-locked outputs (cudaHostAlloc / cudaHostRegister) are
 * written by the kernels directly over the host link while the rays are traced; pageable outputs go
 * through the library's own device buffers and are copied back before the call returns. */
bhk_status bhk_trace_frames_host(bhk_context* ctx, const bhk_frame_desc* frames, int32_t nframes,
                                 const bhk_trace_opts* opts, const bhk_rays_out* host_out);
/* Per-ray variant: explicit (a, r_obs, theta_obs, alpha, beta) device arrays of n rays, ZAMO pinhole
 * launch per ray, shared disk radii (r_disk_in <= 0: each ray's prograde ISCO). */
bhk_status bhk_trace_rays(bhk_context* ctx, int64_t n, const double* a, const double* r_obs, const double* theta_obs,
                          const double* alpha, const double* beta, double r_disk_in, double r_disk_out,
                          const bhk_trace_opts* opts, const bhk_rays_out* out, void* stream);
/* Traces selected pixels of frames: pixels[0..n) are global pixel indices (device memory, int32) over
 * the frames' concatenated row-major pixels, as bhk_trace_frames numbers them; outputs are compact
 * (entry i belongs to pixels[i]). Re-traces and spot checks of rendered images (no counterpart in
 * the reference, whose renderers always trace every pixel). */
bhk_status bhk_trace_pixels(bhk_context* ctx, const bhk_frame_desc* frames, int32_t nframes, const int32_t* pixels,
                            int64_t n, const bhk_trace_opts* opts, const bhk_rays_out* out, void* stream);
/* ---- trajectory::predict (src/trajectory.h:45-57): massive particles (mu = 1) in coordinate time ---- */
enum { BHK_FATE_BOUND = 0, BHK_FATE_CIRCULAR = 1, BHK_FATE_PLUNGES = 2, BHK_FATE_ESCAPES = 3,
       BHK_FATE_HITS_SURFACE = 4 };  /* trajectory::Fate */
typedef struct bhk_path_out {       /* trajectory::Path per particle; NULL members are not written */
    int32_t* fate;                  /* BHK_FATE_* within the time simulated */
    double* duration;               /* coordinate time covered */
    double *r_min, *r_max;
    int32_t* periapses;             /* periapsis passages seen */
    double* precession_deg;         /* periapsis advance per radial period (if periapses >= 2), else 0 */
    double* points;                 /* (max_points + 1) x 3 Kerr-Schild Cartesian points per particle */
    int32_t* n_points;              /* points written (at most max_points + 1: the last is the end) */
} bhk_path_out;
/* trajectory::predict batched: n particles (constants c[i], states s[i], device memory) integrated
 * forward in coordinate time with the reference's own scheme (kerr::stepCoordinateTime at
 * kerr::suggestedTimeStep tolerance 0.01, src/trajectory.cpp:130-185) up to max_time, or until they
 * plunge (horizon, or the surface of radius `surface` if nonzero) or escape past escape_radius;
 * path points at least min_spacing apart (max_points >= 1; the start and the end always count, so a
 * particle writes at most max_points + 1). s_out (may be NULL) receives the final states. FP64. */
bhk_status bhk_predict(double a, const bhk_constants* c, const bhk_state* s, int64_t n, double max_time,
                       double min_spacing, int32_t max_points, double surface, double escape_radius,
                       bhk_state* s_out, const bhk_path_out* out, void* stream);

/* Per-ray cameras with arbitrary frames -- the call shape of trajectory::traceRay(a, r, theta, phi,
 * frame, look, scene) (src/trajectory.h:118-119), batched: camera position (a, r, theta, phi), its
 * frame (kerr::observerFrame of any 4-velocity: ZAMO, boosted, geodesic; bhk_observer_frame builds
 * them) and a unit look direction on the frame's (r, theta, phi) axes (3 doubles per ray), all device
 * memory. Cameras may be inside the horizon: there a photon with 2 r_+ E - a L < 0 ends captured at
 * once (src/trajectory.cpp:236-244), the others are traced back out through r_+. Disk radii as in
 * bhk_trace_rays. */
bhk_status bhk_trace_rays_framed(bhk_context* ctx, int64_t n, const double* a, const double* r, const double* theta,
                                 const double* phi, const bhk_frame* frames, const double* look, double r_disk_in,
                                 double r_disk_out, const bhk_trace_opts* opts, const bhk_rays_out* out,
                                 void* stream);
bhk_status bhk_get_stats(bhk_context* ctx, bhk_trace_stats* stats);   /* synchronises the context stream */
/* Times block x chunk x sort-granularity candidates on these frames and keeps the fastest for later
 * calls on this context (opts fields left 0). The chosen values are returned in stats. */
bhk_status bhk_autotune(bhk_context* ctx, const bhk_frame_desc* frames, int32_t nframes, const bhk_trace_opts* opts,
                        bhk_trace_stats* chosen);

/* Analytic shadow edge seen by a frame's pinhole: spherical photon orbits r in [r_pro, r_retro],
 * their (xi, eta) mapped through the ZAMO camera at r_obs (src/eht.cpp:52-80 for r_obs -> infinity).
 * Host outputs alpha, beta (cap entries); returns the count in *n. */
bhk_status bhk_critical_curve(double a, double r_obs, double theta_obs, int32_t samples, double* alpha, double* beta,
                              int32_t cap, int32_t* n);

/* bhk_trace_frames without any device allocation (no counterpart in the reference). For callers that
 * may not allocate device memory -- a host framework that owns the whole device-memory budget
 * through its own pool, or a per-frame render loop where cudaMalloc/cudaFree would synchronise the
 * device. Outputs are the caller's device buffers (the RayReport extras of bhk_rays_out included);
 * all working memory lives in one fixed array in libbhk's device image (6.1 MB, held by every GPU
 * that loads the library until exit).
 * Frames are checked as bhk_trace_frames checks them (naked singularities, |a| > 1, are traced too).
 * Limits: at most 65536 rays and 64 frames per call; larger requests return BHK_EINVAL. No context:
 * the tracer runs on the current device and on `stream` (NULL = the legacy default stream) with the
 * opts given (0 fields take the context defaults; no autotuning). Asynchronous: BHK_OK means the work
 * is queued, and rays that reach the step cap show only as BHK_RAY_UNFINISHED in `outcome` (this call
 * never returns BHK_EUNFINISHED). All calls share the array, which keeps the previous call's contents
 * (the control block is cleared at the start of each call): calls that overlap on the GPU race, so
 * order them on one stream. The first call on a device (and the first after cudaDeviceReset) looks up
 * the array's device address (cudaGetSymbolAddress); make it before any stream capture. */
bhk_status bhk_trace_frames_static(const bhk_frame_desc* frames, int32_t nframes, const bhk_trace_opts* opts,
                                   const bhk_rays_out* out, void* stream);

/* ---- eht::render (src/eht.h:100-160): the shadow and the synchrotron image of a hot flow ---- */
typedef struct bhk_eht_view {      /* eht::View */
    double a, inclination;         /* spin; inclination (rad) */
    double half_width;             /* the field's half-width (M) */
    int32_t size, pad;             /* pixels across */
    double frequency;              /* Hz */
    double mass_solar;             /* sets the plasma's path lengths */
} bhk_eht_view;
typedef struct bhk_eht_flow {      /* eht::Flow */
    double n0, T0, beta, keplerian, height, sin_theta_b;
} bhk_eht_flow;
/* eht::render: size x size pixels, row-major from beta = +half_width; intensity I_nu (device,
 * double) and shadow (device, 1 where the ray fell in), either may be NULL; steps (device, int32,
 * may be NULL): integration steps per ray. with_light = 0 only follows the rays (the shadow).
 * Asynchronous on `stream` (NULL: the legacy default stream). The image is a sum over eht::traceRay's
 * own steps (src/eht.cpp:260-319), restated in FP64. */
bhk_status bhk_eht_render(const bhk_eht_view* view, const bhk_eht_flow* flow, int32_t with_light, double* intensity,
                          uint8_t* shadow, int32_t* steps, void* stream);
/* eht::flux of a host intensity image: Jy for a source whose M subtends theta_g_uas. */
double bhk_eht_flux(const double* intensity, int32_t size, double half_width, double theta_g_uas);
/* eht::calibrate: the density n0 giving target_jy (secant in log n0 on 48-pixel GPU renders). */
bhk_status bhk_eht_calibrate(const bhk_eht_view* view, const bhk_eht_flow* flow, double target_jy,
                             double theta_g_uas, double* n0);

/* FLOPs one accepted FP32 Dormand-Prince step costs in the mixed tracer, counted from its source. */
double bhk_flops_per_step(void);
/* FLOPs of a rejected FP32 attempt: the same stages, sums and error norm, only the step shrink after. */
double bhk_flops_per_rejected_step(void);

/* Diagnostic: C (M x N, FP32, row-major) = A (M x K) * B (N x K)^T, A and B BF16 row-major in device
 * memory, on the surrogate's tcgen05 GEMM kernel (TMA, TMEM accumulator). N <= 256, K % 8 == 0.
 * splits > 1 splits K across CTAs and accumulates into C atomically (zero C first). Synchronous. */
bhk_status bhk_tc_gemm(const void* A, const void* B, float* C, int32_t M, int32_t N, int32_t K, int32_t splits,
                       void* stream);

/* ---- Surrogate (no counterpart in the reference: the reference has no learned model) ----
 * A BF16 MLP of the tracer: per ray (a, theta_obs, log10 r_obs, alpha, beta) -> 64 Fourier features
 * -> 4 x (256, SiLU) -> 8 outputs: 3 outcome logits (captured, disk, escaped), r_disk / 30, ln g and
 * the unit escape direction (sin th cos ph, sin th sin ph, cos th) of (theta_inf, phi_inf). Trained and
 * run by hand-written tcgen05 kernels (BF16 operands, FP32 accumulation, FP32 master weights and
 * Adam state). Inputs are FP32 [n x 5] rows in device memory; class labels are 1/2/3 (the
 * bhk_ray_outcome values), targets FP32 [n x 8] rows in the output convention above. */
typedef struct bhk_surrogate bhk_surrogate;
int64_t bhk_surrogate_num_params(void);   /* of the default network (hidden width 256) */
/* max_batch: rows of every activation buffer (a multiple of 128). Seeded initialisation. Hidden
 * width 256. */
bhk_status bhk_surrogate_create(int device, uint64_t seed, int32_t max_batch, bhk_surrogate** out);
/* The same network with hidden width 64 or 256 (every other size and layer is unchanged): width 64
 * costs 34,816 FLOPs per ray to evaluate against 434,176, for a coarser fit. */
bhk_status bhk_surrogate_create_width(int device, uint64_t seed, int32_t max_batch, int32_t width,
                                      bhk_surrogate** out);
int32_t bhk_surrogate_width(const bhk_surrogate* s);
int64_t bhk_surrogate_param_count(const bhk_surrogate* s);  /* the length of its parameter vector */
bhk_status bhk_surrogate_destroy(bhk_surrogate* s);
/* Copies the FP32 parameter vector out (set = 0) or in (set != 0); host memory. Layout: for each
 * layer W (fan_out x fan_in, row-major) then b; fan (64->H, H->H x 3, H->16 with the head's rows 8..15
 * padding that stays zero), H the hidden width. */
bhk_status bhk_surrogate_params(bhk_surrogate* s, float* host, int32_t set);
/* The Fourier matrix B (32 x 5, host) of the features [sin, cos](2 pi B u): read (set = 0) or
 * replaced (set != 0). It is not trained; the default is seeded (random directions, frequencies
 * 0.1 .. 4 cycles per unit of the normalised input). */
bhk_status bhk_surrogate_fourier(bhk_surrogate* s, float* host, int32_t set);
/* Weights of the loss terms in the gradient (CE, r_disk MSE, ln g MSE, direction MSE; default
 * 1, 10, 10, 10: the regression terms are ~100x smaller than the cross-entropy at the start). */
bhk_status bhk_surrogate_loss_weights(bhk_surrogate* s, const float* w4);
/* Adam moments (host, num_params floats each) and step count, read or restored (set != 0), for
 * checkpoint and resume together with bhk_surrogate_params and bhk_surrogate_fourier. */
bhk_status bhk_surrogate_adam_state(bhk_surrogate* s, float* m, float* v, int64_t* step, int32_t set);
/* Loss terms (host float[4]: cross-entropy, r_disk MSE, ln g MSE, direction MSE, batch means) and the
 * FP32 gradient of their sum (host, num_params) for n rows (n % 128 == 0), without an update. */
bhk_status bhk_surrogate_gradients(bhk_surrogate* s, const float* x, const uint8_t* cls, const float* target,
                                   int32_t n, float* grads, float* loss);
/* steps Adam updates (beta 0.9 / 0.999) on consecutive batches of `batch` rows cycling through the n
 * rows given, with learning rate lr0 * (1 + cos(pi t / steps)) / 2. loss_history (host, 4 x steps
 * floats) may be NULL. Synchronous. */
bhk_status bhk_surrogate_train(bhk_surrogate* s, const float* x, const uint8_t* cls, const float* target, int64_t n,
                               int32_t batch, int64_t steps, float lr0, float* loss_history, void* stream);
/* Network outputs (FP32 [n x 8], device) for n rays, layer by layer. Synchronous. */
bhk_status bhk_surrogate_predict(bhk_surrogate* s, const float* x, int64_t n, float* out, void* stream);

/* The training set of the surrogate: n rays with a uniform on [0, 0.998], theta_obs uniform on
 * [5, 89] deg, log10 r_obs uniform on [log10 20, 3] and (alpha, beta) uniform in a disk of radius 1.5 x
 * the frame's shadow radius (seeded counter-based draws), traced by ctx (opts NULL: mixed precision)
 * with a disk from each ray's prograde ISCO to r_disk_out, and written as inputs x [n x 5], classes and
 * targets [n x 8] (device memory, the bhk_surrogate_train convention). rays5 (device, 5 x n doubles:
 * a, r_obs, theta_obs, alpha, beta) receives the rays when not NULL. Synchronous. */
bhk_status bhk_surrogate_dataset(bhk_context* ctx, int64_t n, uint64_t seed, double r_disk_out,
                                 const bhk_trace_opts* opts, float* x, uint8_t* cls, float* target, double* rays5,
                                 void* stream);

/* Which of the network's answers a render keeps. BHK_ACCEPT_ALL: every confident ray outside the
 * band (the network's r_disk, g and escape direction are its answers, ~1e-2 accurate). BHK_ACCEPT_CAPTURED:
 * only rays the network classes captured; every disk or escaping ray is traced. A captured ray has no
 * continuous output, so each accepted answer is exactly the tracer's wherever the class is right. */
enum { BHK_ACCEPT_ALL = 0, BHK_ACCEPT_CAPTURED = 1 };

typedef struct bhk_render_opts {
    double p_min;        /* rays whose largest class probability is below this fall back (0.99) */
    double band;         /* rays within this image-plane distance (M) of the critical curve fall back (0.05) */
    int32_t fallback;    /* 1: trace the fallback rays (the product); 0: only list them (measurement) */
    int32_t accept;      /* BHK_ACCEPT_ALL (0) or BHK_ACCEPT_CAPTURED */
} bhk_render_opts;

typedef struct bhk_render_stats {
    int64_t rays, fallback;  /* rays rendered, rays handed to the integrator */
    double infer_ms;         /* fused inference kernel (CUDA events) */
    double trace_ms;         /* fallback trace incl. its launch and the scatter (CUDA events) */
    int32_t accept, grid;    /* the acceptance mode used; CTAs of the inference kernel */
} bhk_render_stats;

/* Renders frames with the surrogate and integrator fallback: one fused tcgen05 inference kernel over
 * every pixel (inputs from the frame table; outputs in the bhk_rays_out convention with phi_disk NaN
 * and steps 0 where the network answered), then the mixed/FP64 tracer (opts) on the fallback list:
 * rays with max class probability < p_min, within `band` of the analytic critical curve, in the
 * axis-snap strip (|alpha| sin(theta_obs) < 4e-3) or with a non-finite output. Outputs are device
 * memory for all pixels (outcome required). ctx supplies the tracer; both on one device. Synchronous.
 * opts and ropts may be NULL (defaults). */
bhk_status bhk_surrogate_render(bhk_surrogate* s, bhk_context* ctx, const bhk_frame_desc* frames, int32_t nframes,
                                const bhk_trace_opts* opts, const bhk_render_opts* ropts, const bhk_rays_out* out,
                                bhk_render_stats* stats, void* stream);
/* The fallback list of the last render: its length in *n, and up to cap global pixel indices (in no
 * particular order) copied into the device buffer dst. */
bhk_status bhk_surrogate_fallback_list(bhk_surrogate* s, int32_t* dst, int64_t cap, int64_t* n);

/* Diagnostic: the device's FP32 FMA throughput (TFLOP/s, FMA = 2 FLOPs) measured with a
 * latency-covered FMA chain kernel, the roofline denominator of the tracer. No reference counterpart. */
bhk_status bhk_fp32_fma_peak(int device, double* tflops);

#ifdef __cplusplus
}
#endif
#endif
