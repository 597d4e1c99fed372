// bhk_api.cu -- host side of libbhk: the C ABI declared in include/bhk.h.
//
// A bhk_context owns a stream, grow-only device scratch (launch records, sort order, rescue list,
// control block), pinned staging for frame descriptors and statistics, the autotuned launch
// shape and a cached CUDA graph of the whole batch pipeline. Frame descriptors and the ray count
// travel through device memory, so one instantiated graph replays any batch that fits the
// scratch capacity without re-capture.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "bhk_internal.h"

using namespace bhk;

namespace {

thread_local std::string g_last_error;

bhk_status fail(bhk_status s, const std::string& msg) {
    g_last_error = msg;
    return s;
}

bhk_status cuda_fail(cudaError_t e, const char* what) {
    return fail(BHK_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define BHK_CUDA(call)                                          \
    do {                                                        \
        cudaError_t e_ = (call);                                \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);     \
    } while (0)

template <typename T>
cudaError_t grow(T** p, size_t* cap, size_t need) {
    if (need <= *cap && *p) return cudaSuccess;
    if (*p) cudaFree(*p);
    *p = nullptr;
    size_t n = std::max<size_t>(need, 1);
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), n * sizeof(T));
    *cap = e == cudaSuccess ? n : 0;
    return e;
}

struct GraphKey {
    int mode = -1, fp64 = 0, nframes = 0, block = 0, chunk = 0, buckets = 0, grid = 0, timed = 0, regcap = 0;
    int64_t n_explicit = 0;
    TraceParams p{};
    Outputs out{};
    const void* ex[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    double r_in = 0.0, r_out = 0.0;
    size_t cap_rays = 0;
    bool operator==(const GraphKey& o) const { return std::memcmp(this, &o, sizeof(GraphKey)) == 0; }
};

// FP32 FLOPs of one Dormand-Prince attempt of the mixed tracer, counted from the source (an FMA is 2):
//   right-hand side (bhk_device.cuh rhs<float>): sine/cosine 23 (10 FMA, 2 MUL, 1 ADD), Delta and
//     r^2 + a^2 4, P 2, inflow 4, sin cos, sin^2 and L / sin^2 3, dphi 4, R'/2 4, Theta'/2 3 -> 47,
//     x 6 stages = 282;
//     the FSAL stage's constraint potentials 15;
//   stage sums y + h sum_j a_ij k_j over 5 components (bhk_trace.cu stage_f32): per stage of M terms
//     and component a product, M - 1 FMA and the FMA by h, 2M + 1 -> 5 x (2 x 20 + 6) = 230;
//   error estimate and weighted norm: 5 x 16 + 2 = 82;  step control and pole cap: 8.
// A rejected attempt does the same stages, sums and norm, then only shrinks the step (3 products).
constexpr double kFlopsPerStep = 617.0;
constexpr double kFlopsPerRejected = 282.0 + 15.0 + 230.0 + 82.0 + 3.0;

}  // namespace

void bhk::set_last_error(const std::string& msg) { g_last_error = msg; }

struct bhk_context {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t capture_stream = nullptr;
    std::mutex mu;

    // scratch
    size_t cap_rays = 0, cap_E = 0, cap_L = 0, cap_Q = 0, cap_vr = 0, cap_vth = 0, cap_gid = 0,
           cap_key = 0, cap_order = 0, cap_rescue = 0, cap_geom = 0, cap_frames = 0;
    double *E = nullptr, *L = nullptr, *Q = nullptr, *vr = nullptr, *vth = nullptr;
    int32_t* gid = nullptr;
    uint16_t* key = nullptr;
    float4* cf = nullptr;
    float2* vf = nullptr;
    float4* kf = nullptr;
    float2* khf = nullptr;
    size_t cap_cf = 0, cap_vf = 0, cap_kf = 0, cap_khf = 0;
    int32_t* order = nullptr;
    Rescue* rescue = nullptr;
    RayGeom* geom = nullptr;
    FrameDev* frames_dev = nullptr;
    Control* ctl = nullptr;
    unsigned* hist = nullptr;
    unsigned* offs = nullptr;

    // pinned staging
    FrameDev* frames_host = nullptr;
    RayGeom* geom_host = nullptr;  // the frames' geometries, set up on the host with the frame table
    size_t cap_frames_host = 0;
    Control* ctl_host = nullptr;
    long long* n_host = nullptr;
    cudaEvent_t staging_free = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool timed_last = false;

    // library-owned outputs for the host-buffer entry point and the autotuner
    size_t cap_out = 0, cap_o8 = 0, cap_od[12] = {}, cap_os = 0, cap_or = 0;
    uint8_t* o_outcome = nullptr;
    double* o_d[12] = {};  // r_disk, phi_disk, g, theta_inf, phi_inf, then the optional seven
    int32_t* o_steps = nullptr;
    int32_t* o_rej = nullptr;

    // launch shape: autotuned per precision, else defaults
    int tuned_block[2] = {0, 0}, tuned_chunk[2] = {0, 0}, tuned_buckets[2] = {0, 0}, tuned_regcap[2] = {0, 0};

    // cached graph
    GraphKey gkey;
    cudaGraphExec_t exec = nullptr;
    cudaGraph_t graph = nullptr;

    bhk_trace_stats last{};
};

namespace {

struct Resolved {
    bool fp64;
    TraceParams p;
    int block, chunk, buckets, grid, regcap;
    bool graph;
};

Resolved resolve(bhk_context* ctx, const bhk_trace_opts* o) {
    bhk_trace_opts d{};
    if (!o) o = &d;
    Resolved r{};
    r.fp64 = o->precision == BHK_PREC_FP64;
    const int pi = r.fp64 ? 0 : 1;
    r.p.rtol = o->rtol > 0.0 ? o->rtol : (r.fp64 ? 1e-10 : 1e-6);
    r.p.eps = o->capture_eps > 0.0 ? o->capture_eps : 1e-6;
    r.p.r_escape = o->r_escape > 0.0 ? o->r_escape : 1000.0;
    r.p.max_steps = o->max_steps > 0 ? o->max_steps : 20000;
    r.p.reproject_every = o->reproject_every > 0 ? o->reproject_every : 0;
    r.p.tol0 = std::min(std::max(std::pow(r.p.rtol, 0.2), 1e-3), 0.05);
    r.p.rtol_f = static_cast<float>(r.p.rtol);
    // Near the Mino-time pole of an outgoing ray the 4th-order error estimate grows as (h / d)^5,
    // d the Mino time left; measured, it allows h / d ~ 0.12 at rtol 1e-6, scaling as rtol^(1/5).
    // The cap sits just below, where the controller would otherwise cycle into rejections (on the
    // a = 0.9, r_obs = 50 frame: 31% rejected steps uncapped, 6% at 0.1, 20% less work in all).
    r.p.pole_frac = o->pole_step_frac > 0.0 ? static_cast<float>(o->pole_step_frac)
                    : (o->pole_step_frac < 0.0 ? 0.0f
                       : static_cast<float>(std::min(0.5, 0.1 * std::pow(r.p.rtol / 1e-6, 0.2))));
    r.p.tol0_f = static_cast<float>(r.p.tol0);
    r.block = o->block > 0 ? o->block : (ctx->tuned_block[pi] ? ctx->tuned_block[pi] : 128);
    r.chunk = o->chunk > 0 ? o->chunk : (ctx->tuned_chunk[pi] ? ctx->tuned_chunk[pi] : 32);
    r.chunk = (std::max(r.chunk, 32) + 31) / 32 * 32;  // whole batches of 32 (one per lane)
    r.buckets = o->sort_buckets > 0 ? o->sort_buckets : (ctx->tuned_buckets[pi] ? ctx->tuned_buckets[pi] : 1);
    r.buckets = std::min(r.buckets, kMaxBuckets);
    r.p.chunk = r.chunk;
    r.p.buckets = r.buckets;
    r.graph = o->use_graph != 0;
    const int rb = o->reg_budget > 0 ? o->reg_budget : (ctx->tuned_regcap[pi] ? ctx->tuned_regcap[pi] : 1);
    r.regcap = (r.fp64 || rb >= 3) ? 0 : rb;
    r.p.fp64_turning = (!r.fp64 && o->fp64_turning) ? 1 : 0;
    if (r.p.fp64_turning) r.regcap = 1;  // the variant with FP64 turning-point attempts is built at <= 102
    if (r.regcap > 0 && r.block > 128) r.block = 128;
    r.block = std::min(r.block, 256);
    const int bps = trace_blocks_per_sm(r.fp64, r.regcap, r.block);
    r.grid = std::max(1, bps) * ctx->num_sms;
    return r;
}

bhk_status ensure_scratch(bhk_context* c, size_t rays, size_t geoms, size_t frames) {
    const size_t rc = rays / 4 + 4096;
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = grow(&c->E, &c->cap_E, rays);
    if (e == cudaSuccess) e = grow(&c->L, &c->cap_L, rays);
    if (e == cudaSuccess) e = grow(&c->Q, &c->cap_Q, rays);
    if (e == cudaSuccess) e = grow(&c->vr, &c->cap_vr, rays);
    if (e == cudaSuccess) e = grow(&c->vth, &c->cap_vth, rays);
    if (e == cudaSuccess) e = grow(&c->gid, &c->cap_gid, rays);
    if (e == cudaSuccess) e = grow(&c->key, &c->cap_key, rays);
    if (e == cudaSuccess) e = grow(&c->cf, &c->cap_cf, rays);
    if (e == cudaSuccess) e = grow(&c->vf, &c->cap_vf, rays);
    if (e == cudaSuccess) e = grow(&c->kf, &c->cap_kf, rays);
    if (e == cudaSuccess) e = grow(&c->khf, &c->cap_khf, rays);
    if (e == cudaSuccess) e = grow(&c->order, &c->cap_order, rays);
    if (e == cudaSuccess) e = grow(&c->rescue, &c->cap_rescue, rc);
    if (e == cudaSuccess) e = grow(&c->geom, &c->cap_geom, geoms);
    if (e == cudaSuccess) e = grow(&c->frames_dev, &c->cap_frames, frames);
    if (e != cudaSuccess) return fail(BHK_ENOMEM, std::string("scratch allocation: ") + cudaGetErrorString(e));
    c->cap_rays = std::min({c->cap_E, c->cap_order, c->cap_key, c->cap_cf, c->cap_vf, c->cap_kf, c->cap_khf});
    if (frames > c->cap_frames_host) {
        if (c->frames_host) cudaFreeHost(c->frames_host);
        if (c->geom_host) cudaFreeHost(c->geom_host);
        c->frames_host = nullptr;
        c->geom_host = nullptr;
        c->cap_frames_host = 0;
        e = cudaMallocHost(reinterpret_cast<void**>(&c->frames_host), frames * sizeof(FrameDev));
        if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&c->geom_host), frames * sizeof(RayGeom));
        if (e != cudaSuccess) return fail(BHK_ENOMEM, "pinned staging allocation");
        c->cap_frames_host = frames;
    }
    return BHK_OK;
}

LaunchSoA soa(bhk_context* c) {
    return LaunchSoA{c->E, c->L, c->Q, c->vr, c->vth, c->gid, c->key, c->cf, c->vf, c->kf, c->khf};
}

struct Batch {
    int mode;  // 0 frames, 1 explicit, 2 a list of pixels of the frames (ex[0] = the device list),
               // 3 framed cameras (ex = a, r, theta, phi, frames, look)
    int nframes;
    int64_t n;
    const double* ex[6];
    double r_in, r_out;
};

// Enqueues the whole pipeline on stream s (also used while capturing a graph).
bhk_status enqueue(bhk_context* c, const Batch& b, const Resolved& r, const Outputs& out, bool timed,
                   cudaStream_t s) {
    BHK_CUDA(cudaMemsetAsync(c->ctl, 0, sizeof(Control), s));
    const int lgrid = c->num_sms * 8;
    LaunchSoA L = soa(c);
    if (r.fp64) {  // the FP32 start is for the FP32 tracer only
        L.kf = nullptr;
        L.khf = nullptr;
    }
    if (b.mode == 0 || b.mode == 2) {  // the frame table, its geometries and the ray count, set up on the host
        BHK_CUDA(cudaMemcpyAsync(c->frames_dev, c->frames_host, sizeof(FrameDev) * b.nframes, cudaMemcpyHostToDevice,
                                 s));
        BHK_CUDA(cudaMemcpyAsync(c->geom, c->geom_host, sizeof(RayGeom) * b.nframes, cudaMemcpyHostToDevice, s));
        BHK_CUDA(cudaMemcpyAsync(&c->ctl->n_rays, c->n_host, sizeof(long long), cudaMemcpyHostToDevice, s));
    }
    if (b.mode == 0) {
        // With the cost sort the keys are needed first; otherwise the trace kernel launches the rays.
        if (r.buckets > 1) launch_rays_frames(c->frames_dev, c->geom, b.nframes, L, r.p, c->ctl, lgrid, s);
    } else if (b.mode == 2) {  // the batch is the list (its length staged as the ray count)
        launch_rays_list(c->frames_dev, c->geom, b.nframes,
                         static_cast<const int32_t*>(static_cast<const void*>(b.ex[0])), L, r.p, c->ctl, lgrid, s);
    } else if (b.mode == 3) {
        BHK_CUDA(cudaMemcpyAsync(&c->ctl->n_rays, c->n_host, sizeof(long long), cudaMemcpyHostToDevice, s));
        launch_rays_framed(b.ex[0], b.ex[1], b.ex[2], b.ex[3], reinterpret_cast<const bhk_frame*>(b.ex[4]), b.ex[5],
                           b.r_in, b.r_out, c->geom, L, r.p, c->ctl, lgrid, s);
    } else {
        BHK_CUDA(cudaMemcpyAsync(&c->ctl->n_rays, c->n_host, sizeof(long long), cudaMemcpyHostToDevice, s));
        launch_rays_explicit(b.ex[0], b.ex[1], b.ex[2], b.ex[3], b.ex[4], b.r_in, b.r_out, c->geom, L, r.p, c->ctl,
                             lgrid, s);
    }
    const int32_t* order = nullptr;
    if (r.buckets > 1) {
        BHK_CUDA(cudaMemsetAsync(c->hist, 0, sizeof(unsigned) * kMaxBuckets, s));
        launch_sort(L, SortScratch{c->hist, c->offs, c->order}, r.p, c->ctl, lgrid, s);
        order = c->order;
    }  // frames without the sort: the trace kernel takes its rays by 8 x 4 pixel tiles itself
    if (timed) BHK_CUDA(cudaEventRecord(c->ev0, s));
    const bool fused = b.mode == 0 && r.buckets <= 1;
    launch_trace(r.fp64, r.regcap, L, c->geom, order, out, c->rescue, static_cast<unsigned>(c->cap_rescue), r.p, c->ctl,
                 r.block, r.grid, s, fused ? c->frames_dev : nullptr, fused ? b.nframes : 0);
    if (!r.fp64)
        launch_rescue(L, c->geom, out, c->rescue, static_cast<unsigned>(c->cap_rescue), r.p, c->ctl, c->num_sms, s);
    if (timed) BHK_CUDA(cudaEventRecord(c->ev1, s));
    launch_constants_out(L, out, c->ctl, lgrid, s);
    BHK_CUDA(cudaMemcpyAsync(c->ctl_host, c->ctl, sizeof(Control), cudaMemcpyDeviceToHost, s));
    BHK_CUDA(cudaGetLastError());
    return BHK_OK;
}

bhk_status run_batch(bhk_context* c, const Batch& b, const Resolved& r, const Outputs& out, bool timed,
                     cudaStream_t s) {
    if (!r.graph) return enqueue(c, b, r, out, timed, s);
    // In a graph the timing events bracket the whole replay, recorded on the launching stream:
    // events recorded inside a captured graph cannot be read back with cudaEventElapsedTime.
    GraphKey k;
    std::memset(static_cast<void*>(&k), 0, sizeof(GraphKey));  // padding takes part in the comparison
    k.mode = b.mode; k.fp64 = r.fp64; k.nframes = b.nframes; k.block = r.block; k.chunk = r.chunk;
    k.buckets = r.buckets; k.grid = r.grid; k.timed = 0; k.regcap = r.regcap; k.p = r.p; k.out = out; k.cap_rays = c->cap_rays;
    k.n_explicit = b.mode != 0 ? 1 : 0;
    for (int i = 0; i < 6; ++i) k.ex[i] = b.ex[i];
    k.r_in = b.r_in; k.r_out = b.r_out;
    if (!c->exec || !(k == c->gkey)) {
        if (c->exec) cudaGraphExecDestroy(c->exec);
        if (c->graph) cudaGraphDestroy(c->graph);
        c->exec = nullptr;
        c->graph = nullptr;
        BHK_CUDA(cudaStreamBeginCapture(c->capture_stream, cudaStreamCaptureModeThreadLocal));
        const bhk_status st = enqueue(c, b, r, out, false, c->capture_stream);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(c->capture_stream, &g);
        if (st != BHK_OK) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
        c->graph = g;
        BHK_CUDA(cudaGraphInstantiate(&c->exec, g, 0));
        c->gkey = k;
    }
    if (timed) BHK_CUDA(cudaEventRecord(c->ev0, s));
    BHK_CUDA(cudaGraphLaunch(c->exec, s));
    if (timed) BHK_CUDA(cudaEventRecord(c->ev1, s));
    return BHK_OK;
}

Outputs to_outputs(const bhk_rays_out* o) {
    Outputs r{};
    if (!o) return r;
    r.outcome = o->outcome; r.r_disk = o->r_disk; r.phi_disk = o->phi_disk; r.g = o->g;
    r.theta_inf = o->theta_inf; r.phi_inf = o->phi_inf; r.steps = o->steps; r.rejected = o->rejected;
    r.energy = o->energy; r.g_camera = o->g_camera; r.b = o->b; r.q = o->q; r.r_min = o->r_min;
    r.delay = o->delay; r.turns = o->turns;
    return r;
}

bhk_status check_frames(const bhk_frame_desc* f, int32_t nframes, int64_t* total) {
    if (!f || nframes <= 0) return fail(BHK_EINVAL, "frames: null pointer or nframes <= 0");
    int64_t t = 0;
    for (int i = 0; i < nframes; ++i) {
        if (f[i].width <= 0 || f[i].height <= 0) return fail(BHK_EINVAL, "frame with non-positive size");
        // |a| > 1 is a naked singularity (no horizon); the extremal |a| = 1 is refused.
        const double aa = std::fabs(f[i].a);
        if (!(aa < 1.0 || aa > 1.0)) return fail(BHK_EINVAL, "spin must be finite and |a| != 1");
        const double rp = aa < 1.0 ? 1.0 + std::sqrt(1.0 - f[i].a * f[i].a) : 0.0;
        if (!(f[i].r_obs > rp))
            return fail(BHK_EINVAL, "camera must sit outside the horizon (ZAMO pinhole; r_obs > 0 past |a| = 1)");
        if (!(f[i].theta_obs > 0.0 && f[i].theta_obs < M_PI)) return fail(BHK_EINVAL, "theta_obs outside (0, pi)");
        if (!(f[i].r_disk_out >= 0.0)) return fail(BHK_EINVAL, "r_disk_out must be >= 0 (0: no disk)");
        t += static_cast<int64_t>(f[i].width) * f[i].height;
    }
    if (t > (int64_t(1) << 31) - 1) return fail(BHK_EINVAL, "more than 2^31 - 1 rays in one batch");
    *total = t;
    return BHK_OK;
}

// Fills the pinned frame table, the frames' geometries and the ray count (the FP64 per-frame set-up
// runs here, on the host, while the previous batch may still be tracing).
bhk_status stage_frames(bhk_context* c, const bhk_frame_desc* f, int32_t nframes, const TraceParams& p) {
    // The previous batch's H2D copy may still read the staging buffers.
    if (c->staging_free) BHK_CUDA(cudaEventSynchronize(c->staging_free));
    for (int i = 0; i < nframes; ++i) {
        std::memset(&c->frames_host[i], 0, sizeof(FrameDev));
        std::memset(&c->geom_host[i], 0, sizeof(RayGeom));
        c->frames_host[i].d = f[i];
    }
    *c->n_host = setup_frames_host(c->frames_host, c->geom_host, nframes, p);
    return BHK_OK;
}

bhk_status finish_call(bhk_context* c, const Resolved& r, int64_t n, bool timed, cudaStream_t s) {
    BHK_CUDA(cudaEventRecord(c->staging_free, s));
    c->last = bhk_trace_stats{};
    c->last.rays = n;
    c->last.block = r.block;
    c->last.chunk = r.chunk;
    c->last.sort_buckets = r.buckets;
    c->last.grid = r.grid;
    c->last.reg_budget = r.fp64 ? 0 : (r.regcap ? r.regcap : 3);
    c->timed_last = timed;
    return BHK_OK;
}

bhk_status ensure_outputs(bhk_context* c, size_t n, bool extras = false) {
    cudaError_t e = grow(&c->o_outcome, &c->cap_o8, n);
    for (int i = 0; i < (extras ? 12 : 5) && e == cudaSuccess; ++i) e = grow(&c->o_d[i], &c->cap_od[i], n);
    if (e == cudaSuccess) e = grow(&c->o_steps, &c->cap_os, n);
    if (e == cudaSuccess) e = grow(&c->o_rej, &c->cap_or, n);
    if (e != cudaSuccess) return fail(BHK_ENOMEM, "output allocation");
    return BHK_OK;
}

bhk_rays_out own_outputs(bhk_context* c) {
    bhk_rays_out o{};
    o.outcome = c->o_outcome;
    o.r_disk = c->o_d[0]; o.phi_disk = c->o_d[1]; o.g = c->o_d[2]; o.theta_inf = c->o_d[3]; o.phi_inf = c->o_d[4];
    o.steps = c->o_steps; o.rejected = c->o_rej;
    return o;
}

cudaStream_t pick(bhk_context* c, void* stream) { return stream ? static_cast<cudaStream_t>(stream) : c->stream; }

bhk_status trace_frames_locked(bhk_context* c, const bhk_frame_desc* frames, int32_t nframes,
                               const bhk_trace_opts* opts, const bhk_rays_out* out, cudaStream_t s, bool timed) {
    int64_t total = 0;
    bhk_status st = check_frames(frames, nframes, &total);
    if (st != BHK_OK) return st;
    if (!out) return fail(BHK_EINVAL, "out is null");
    st = ensure_scratch(c, static_cast<size_t>(total), static_cast<size_t>(nframes), static_cast<size_t>(nframes));
    if (st != BHK_OK) return st;
    const Resolved r = resolve(c, opts);
    st = stage_frames(c, frames, nframes, r.p);
    if (st != BHK_OK) return st;
    Batch b{0, nframes, total, {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr}, 0.0, 0.0};
    st = run_batch(c, b, r, to_outputs(out), timed, s);
    if (st != BHK_OK) return st;
    return finish_call(c, r, total, timed, s);
}

}  // namespace

bhk_status bhk::validate_frames(const bhk_frame_desc* f, int32_t nframes, int64_t* total) {
    return check_frames(f, nframes, total);
}

bhk_status bhk::trace_pixel_list(bhk_context* c, const bhk_frame_desc* frames, int32_t nframes, const int32_t* list,
                                 int64_t n, const bhk_trace_opts* opts, const bhk_rays_out* out, bhk_rays_out* used,
                                 cudaStream_t s) {
    int64_t total = 0;
    bhk_status st = check_frames(frames, nframes, &total);
    if (st != BHK_OK) return st;
    if (n < 0 || n > total) return fail(BHK_EINVAL, "pixel count out of range");
    if (n > 0 && !list) return fail(BHK_EINVAL, "pixel list is null");
    bhk_rays_out o{};
    if (out) {
        o = *out;
    } else {
        st = ensure_outputs(c, static_cast<size_t>(std::max<int64_t>(n, 1)));
        if (st != BHK_OK) return st;
        o = own_outputs(c);
    }
    if (used) *used = o;
    if (n == 0) return BHK_OK;
    st = ensure_scratch(c, static_cast<size_t>(n), static_cast<size_t>(nframes), static_cast<size_t>(nframes));
    if (st != BHK_OK) return st;
    const Resolved r = resolve(c, opts);
    st = stage_frames(c, frames, nframes, r.p);  // also waits until the pinned ray count is free
    if (st != BHK_OK) return st;
    *c->n_host = n;
    Batch b{2, nframes, n, {reinterpret_cast<const double*>(list), nullptr, nullptr, nullptr, nullptr, nullptr},
            0.0, 0.0};
    st = run_batch(c, b, r, to_outputs(&o), true, s);
    if (st != BHK_OK) return st;
    return finish_call(c, r, n, true, s);
}

std::mutex& bhk::context_mutex(bhk_context* c) { return c->mu; }
cudaStream_t bhk::context_stream(bhk_context* c, void* stream) { return pick(c, stream); }
int bhk::context_device(bhk_context* c) { return c->device; }

extern "C" {

bhk_status bhk_trace_pixels(bhk_context* c, const bhk_frame_desc* frames, int32_t nframes, const int32_t* pixels,
                            int64_t n, const bhk_trace_opts* opts, const bhk_rays_out* out, void* stream) {
    if (!c) return fail(BHK_EINVAL, "context is null");
    if (!out) return fail(BHK_EINVAL, "out is null");
    std::lock_guard<std::mutex> lock(c->mu);
    BHK_CUDA(cudaSetDevice(c->device));
    return trace_pixel_list(c, frames, nframes, pixels, n, opts, out, nullptr, pick(c, stream));
}

const char* bhk_last_error(void) { return g_last_error.c_str(); }
const char* bhk_version(void) { return "bhk 0.1 (sm_103a)"; }
double bhk_flops_per_step(void) { return kFlopsPerStep; }
double bhk_flops_per_rejected_step(void) { return kFlopsPerRejected; }

bhk_status bhk_create(int device, bhk_context** out) {
    if (!out) return fail(BHK_EINVAL, "out is null");
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) return fail(BHK_ECUDA, "no CUDA device (libbhk has no CPU fallback)");
    if (device < 0 || device >= count) return fail(BHK_EINVAL, "device index out of range");
    BHK_CUDA(cudaSetDevice(device));
    bhk_context* c = new bhk_context();
    c->device = device;
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->capture_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->staging_free, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&c->ctl), sizeof(Control));
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&c->hist), sizeof(unsigned) * kMaxBuckets);
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&c->offs), sizeof(unsigned) * kMaxBuckets);
    if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&c->ctl_host), sizeof(Control));
    if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&c->n_host), sizeof(long long));
    if (e != cudaSuccess) {
        bhk_destroy(c);
        return cuda_fail(e, "bhk_create");
    }
    std::memset(c->ctl_host, 0, sizeof(Control));
    *out = c;
    return BHK_OK;
}

bhk_status bhk_destroy(bhk_context* c) {
    if (!c) return BHK_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->exec) cudaGraphExecDestroy(c->exec);
    if (c->graph) cudaGraphDestroy(c->graph);
    void* dev[] = {c->E, c->L, c->Q, c->vr, c->vth, c->gid, c->key, c->cf, c->vf, c->order, c->rescue, c->geom,
                   c->frames_dev, c->ctl, c->hist, c->offs, c->o_outcome, c->o_steps, c->o_rej};
    for (void* p : dev)
        if (p) cudaFree(p);
    for (double* p : c->o_d)
        if (p) cudaFree(p);
    if (c->frames_host) cudaFreeHost(c->frames_host);
    if (c->geom_host) cudaFreeHost(c->geom_host);
    if (c->ctl_host) cudaFreeHost(c->ctl_host);
    if (c->n_host) cudaFreeHost(c->n_host);
    if (c->staging_free) cudaEventDestroy(c->staging_free);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c->capture_stream) cudaStreamDestroy(c->capture_stream);
    delete c;
    return BHK_OK;
}

// ---------------------------------------------------------------------- per-step mirrors ----

#define BHK_STEP_CHECK(cond)                                                        \
    do {                                                                            \
        if (n < 0) return fail(BHK_EINVAL, "negative count");                       \
        if (n == 0) return BHK_OK;                                                  \
        if (!(cond)) return fail(BHK_EINVAL, "null array");                         \
    } while (0)

#define BHK_STEP_RUN(expr)                                                          \
    do {                                                                            \
        cudaError_t e_ = (expr);                                                    \
        if (e_ != cudaSuccess) return cuda_fail(e_, #expr);                         \
        return BHK_OK;                                                              \
    } while (0)

bhk_status bhk_derivatives(double a, const bhk_constants* c, const bhk_state* s, bhk_derivatives_t* d, int64_t n,
                           void* stream) {
    BHK_STEP_CHECK(c && s && d);
    BHK_STEP_RUN(steps_derivatives(a, c, s, d, n, static_cast<cudaStream_t>(stream)));
}
bhk_status bhk_step_mino(double a, const bhk_constants* c, bhk_state* s, const double* h, int64_t n, void* stream) {
    BHK_STEP_CHECK(c && s && h);
    BHK_STEP_RUN(steps_step_mino(a, c, s, h, n, static_cast<cudaStream_t>(stream)));
}
bhk_status bhk_photon_step_size(double a, const bhk_constants* c, const bhk_state* s, double tolerance, double* h,
                                int64_t n, void* stream) {
    BHK_STEP_CHECK(c && s && h);
    if (!(tolerance > 0.0)) return fail(BHK_EINVAL, "tolerance must be positive");
    BHK_STEP_RUN(steps_photon_step_size(a, c, s, tolerance, h, n, static_cast<cudaStream_t>(stream)));
}
bhk_status bhk_enforce_constraints(double a, const bhk_constants* c, bhk_state* s, int64_t n, void* stream) {
    BHK_STEP_CHECK(c && s);
    BHK_STEP_RUN(steps_enforce_constraints(a, c, s, n, static_cast<cudaStream_t>(stream)));
}
bhk_status bhk_normalize_angles(bhk_state* s, int64_t n, void* stream) {
    BHK_STEP_CHECK(s);
    BHK_STEP_RUN(steps_normalize_angles(s, n, static_cast<cudaStream_t>(stream)));
}
bhk_status bhk_potentials(double a, const bhk_constants* c, const bhk_state* s, double* R, double* Theta, int64_t n,
                          void* stream) {
    BHK_STEP_CHECK(c && s && (R || Theta));
    BHK_STEP_RUN(steps_potentials(a, c, s, R, Theta, n, static_cast<cudaStream_t>(stream)));
}
bhk_status bhk_observer_frame(double a, const double* r, const double* theta, const double* u, bhk_frame* f,
                              int64_t n, void* stream) {
    BHK_STEP_CHECK(r && theta && f);
    BHK_STEP_RUN(steps_observer_frame(a, r, theta, u, f, n, static_cast<cudaStream_t>(stream)));
}
bhk_status bhk_photon_from_frame(double a, double r, double theta, double phi, const bhk_frame* frame,
                                 const double* look, bhk_constants* c, bhk_state* s, int64_t n, void* stream) {
    BHK_STEP_CHECK(frame && look && c && s);
    BHK_STEP_RUN(steps_photon_from_frame(a, r, theta, phi, frame, look, c, s, n, static_cast<cudaStream_t>(stream)));
}
bhk_status bhk_launch_from_zamo(double a, double r, double theta, double phi, const double* v, double mu,
                                bhk_constants* c, bhk_state* s, int64_t n, void* stream) {
    BHK_STEP_CHECK(v && c && s);
    BHK_STEP_RUN(steps_launch_from_zamo(a, r, theta, phi, v, mu, c, s, n, static_cast<cudaStream_t>(stream)));
}
bhk_status bhk_cartesian_velocity(double a, const bhk_constants* c, const bhk_state* s, double* out, int64_t n,
                                  void* stream) {
    BHK_STEP_CHECK(c && s && out);
    BHK_STEP_RUN(steps_cartesian_velocity(a, c, s, out, n, static_cast<cudaStream_t>(stream)));
}

bhk_status bhk_predict(double a, const bhk_constants* c, const bhk_state* s, int64_t n, double max_time,
                       double min_spacing, int32_t max_points, double surface, double escape_radius,
                       bhk_state* s_out, const bhk_path_out* out, void* stream) {
    if (!c || !s || !out || n < 0 || max_points < 1 || !(max_time >= 0.0) || !(std::fabs(a) < 1.0))
        return fail(BHK_EINVAL, "bhk_predict: bad arguments (|a| < 1, n >= 0, max_points >= 1)");
    if (n == 0) return BHK_OK;
    const cudaError_t e = steps_predict(a, c, s, n, max_time, min_spacing, max_points, surface, escape_radius, s_out,
                                        *out, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "bhk_predict");
    return BHK_OK;
}

// ------------------------------------------------------------------------- batch tracer ----

bhk_status bhk_trace_frames(bhk_context* c, const bhk_frame_desc* frames, int32_t nframes,
                            const bhk_trace_opts* opts, const bhk_rays_out* out, void* stream) {
    if (!c) return fail(BHK_EINVAL, "context is null");
    std::lock_guard<std::mutex> lock(c->mu);
    BHK_CUDA(cudaSetDevice(c->device));
    return trace_frames_locked(c, frames, nframes, opts, out, pick(c, stream), true);
}

bhk_status bhk_trace_frames_host(bhk_context* c, const bhk_frame_desc* frames, int32_t nframes,
                                 const bhk_trace_opts* opts, const bhk_rays_out* host_out) {
    if (!c) return fail(BHK_EINVAL, "context is null");
    if (!host_out) return fail(BHK_EINVAL, "host_out is null");
    std::lock_guard<std::mutex> lock(c->mu);
    BHK_CUDA(cudaSetDevice(c->device));
    int64_t total = 0;
    bhk_status st = check_frames(frames, nframes, &total);
    if (st != BHK_OK) return st;
    double* hx[7] = {host_out->energy, host_out->g_camera, host_out->b, host_out->q, host_out->r_min, host_out->delay,
                     host_out->turns};
    bool extras = false;
    for (double* p : hx) extras = extras || p;
    st = ensure_outputs(c, static_cast<size_t>(total), extras);
    if (st != BHK_OK) return st;
    // Page-locked (or registered) host outputs are written by the kernels themselves, over the host
    // link while the rays are traced; other host memory goes through device buffers and copies.
    {
        void* hp[15] = {host_out->outcome, host_out->r_disk, host_out->phi_disk, host_out->g, host_out->theta_inf,
                        host_out->phi_inf, host_out->steps, host_out->rejected, hx[0], hx[1], hx[2], hx[3], hx[4],
                        hx[5], hx[6]};
        void* dp[15] = {};
        bool all_mapped = true;
        for (int i = 0; i < 15 && all_mapped; ++i) {
            if (!hp[i]) continue;
            cudaPointerAttributes a{};
            if (cudaPointerGetAttributes(&a, hp[i]) != cudaSuccess) {
                cudaGetLastError();
                all_mapped = false;
            } else if (a.type != cudaMemoryTypeHost || !a.devicePointer) {
                all_mapped = false;
            } else {
                dp[i] = a.devicePointer;
            }
        }
        if (all_mapped) {
            bhk_rays_out direct{};
            direct.outcome = static_cast<uint8_t*>(dp[0]);
            direct.r_disk = static_cast<double*>(dp[1]);
            direct.phi_disk = static_cast<double*>(dp[2]);
            direct.g = static_cast<double*>(dp[3]);
            direct.theta_inf = static_cast<double*>(dp[4]);
            direct.phi_inf = static_cast<double*>(dp[5]);
            direct.steps = static_cast<int32_t*>(dp[6]);
            direct.rejected = static_cast<int32_t*>(dp[7]);
            direct.energy = static_cast<double*>(dp[8]);
            direct.g_camera = static_cast<double*>(dp[9]);
            direct.b = static_cast<double*>(dp[10]);
            direct.q = static_cast<double*>(dp[11]);
            direct.r_min = static_cast<double*>(dp[12]);
            direct.delay = static_cast<double*>(dp[13]);
            direct.turns = static_cast<double*>(dp[14]);
            st = trace_frames_locked(c, frames, nframes, opts, &direct, c->stream, true);
            if (st != BHK_OK) return st;
            BHK_CUDA(cudaStreamSynchronize(c->stream));
            return c->ctl_host->stats[2] ? fail(BHK_EUNFINISHED, "some rays reached the step cap") : BHK_OK;
        }
    }
    const bhk_rays_out dev = own_outputs(c);
    bhk_rays_out use{};
    double** ux[7] = {&use.energy, &use.g_camera, &use.b, &use.q, &use.r_min, &use.delay, &use.turns};
    for (int i = 0; i < 7; ++i) *ux[i] = hx[i] ? c->o_d[5 + i] : nullptr;
    use.outcome = host_out->outcome ? dev.outcome : nullptr;
    use.r_disk = host_out->r_disk ? dev.r_disk : nullptr;
    use.phi_disk = host_out->phi_disk ? dev.phi_disk : nullptr;
    use.g = host_out->g ? dev.g : nullptr;
    use.theta_inf = host_out->theta_inf ? dev.theta_inf : nullptr;
    use.phi_inf = host_out->phi_inf ? dev.phi_inf : nullptr;
    use.steps = host_out->steps ? dev.steps : nullptr;
    use.rejected = host_out->rejected ? dev.rejected : nullptr;
    cudaStream_t s = c->stream;
    st = trace_frames_locked(c, frames, nframes, opts, &use, s, true);
    if (st != BHK_OK) return st;
    const size_t n = static_cast<size_t>(total);
    if (host_out->outcome) BHK_CUDA(cudaMemcpyAsync(host_out->outcome, use.outcome, n, cudaMemcpyDeviceToHost, s));
    double* hd[5] = {host_out->r_disk, host_out->phi_disk, host_out->g, host_out->theta_inf, host_out->phi_inf};
    double* dd[5] = {use.r_disk, use.phi_disk, use.g, use.theta_inf, use.phi_inf};
    for (int i = 0; i < 5; ++i)
        if (hd[i]) BHK_CUDA(cudaMemcpyAsync(hd[i], dd[i], n * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (host_out->steps)
        BHK_CUDA(cudaMemcpyAsync(host_out->steps, use.steps, n * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    if (host_out->rejected)
        BHK_CUDA(cudaMemcpyAsync(host_out->rejected, use.rejected, n * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    for (int i = 0; i < 7; ++i)
        if (hx[i]) BHK_CUDA(cudaMemcpyAsync(hx[i], *ux[i], n * sizeof(double), cudaMemcpyDeviceToHost, s));
    BHK_CUDA(cudaStreamSynchronize(s));
    return c->ctl_host->stats[2] ? fail(BHK_EUNFINISHED, "some rays reached the step cap") : BHK_OK;
}

bhk_status bhk_trace_rays(bhk_context* c, int64_t n, const double* a, const double* r_obs, const double* theta_obs,
                          const double* alpha, const double* beta, double r_disk_in, double r_disk_out,
                          const bhk_trace_opts* opts, const bhk_rays_out* out, void* stream) {
    if (!c) return fail(BHK_EINVAL, "context is null");
    if (n < 0 || n > (int64_t(1) << 31) - 1) return fail(BHK_EINVAL, "ray count out of range");
    if (!out) return fail(BHK_EINVAL, "out is null");
    if (n == 0) return BHK_OK;
    if (!a || !r_obs || !theta_obs || !alpha || !beta) return fail(BHK_EINVAL, "null ray array");
    if (!(r_disk_out >= 0.0)) return fail(BHK_EINVAL, "r_disk_out must be >= 0 (0: no disk)");
    std::lock_guard<std::mutex> lock(c->mu);
    BHK_CUDA(cudaSetDevice(c->device));
    bhk_status st = ensure_scratch(c, static_cast<size_t>(n), static_cast<size_t>(n), 1);
    if (st != BHK_OK) return st;
    const Resolved r = resolve(c, opts);
    cudaStream_t s = pick(c, stream);
    if (c->staging_free) BHK_CUDA(cudaEventSynchronize(c->staging_free));
    *c->n_host = n;
    Batch b{1, 0, n, {a, r_obs, theta_obs, alpha, beta, nullptr}, r_disk_in, r_disk_out};
    st = run_batch(c, b, r, to_outputs(out), true, s);
    if (st != BHK_OK) return st;
    return finish_call(c, r, n, true, s);
}

bhk_status bhk_trace_rays_framed(bhk_context* c, int64_t n, const double* a, const double* r, const double* theta,
                                 const double* phi, const bhk_frame* frames, const double* look, double r_disk_in,
                                 double r_disk_out, const bhk_trace_opts* opts, const bhk_rays_out* out,
                                 void* stream) {
    if (!c) return fail(BHK_EINVAL, "context is null");
    if (n < 0 || n > (int64_t(1) << 31) - 1) return fail(BHK_EINVAL, "ray count out of range");
    if (!out) return fail(BHK_EINVAL, "out is null");
    if (n == 0) return BHK_OK;
    if (!a || !r || !theta || !phi || !frames || !look) return fail(BHK_EINVAL, "null ray array");
    if (!(r_disk_out >= 0.0)) return fail(BHK_EINVAL, "r_disk_out must be >= 0 (0: no disk)");
    std::lock_guard<std::mutex> lock(c->mu);
    BHK_CUDA(cudaSetDevice(c->device));
    bhk_status st = ensure_scratch(c, static_cast<size_t>(n), static_cast<size_t>(n), 1);
    if (st != BHK_OK) return st;
    const Resolved rs = resolve(c, opts);
    cudaStream_t s = pick(c, stream);
    if (c->staging_free) BHK_CUDA(cudaEventSynchronize(c->staging_free));
    *c->n_host = n;
    Batch b{3, 0, n, {a, r, theta, phi, reinterpret_cast<const double*>(frames), look}, r_disk_in, r_disk_out};
    st = run_batch(c, b, rs, to_outputs(out), true, s);
    if (st != BHK_OK) return st;
    return finish_call(c, rs, n, true, s);
}

bhk_status bhk_get_stats(bhk_context* c, bhk_trace_stats* stats) {
    if (!c || !stats) return fail(BHK_EINVAL, "null argument");
    std::lock_guard<std::mutex> lock(c->mu);
    BHK_CUDA(cudaSetDevice(c->device));
    if (c->staging_free) BHK_CUDA(cudaEventSynchronize(c->staging_free));
    bhk_trace_stats s = c->last;
    s.accepted_steps = static_cast<int64_t>(c->ctl_host->stats[0]);
    s.rejected_steps = static_cast<int64_t>(c->ctl_host->stats[1]);
    s.unfinished = static_cast<int64_t>(c->ctl_host->stats[2]);
    s.rescued = static_cast<int64_t>(c->ctl_host->stats[3]);
    s.fp64_turning_steps = static_cast<int64_t>(c->ctl_host->stats[4]);
    s.kernel_ms = 0.0;
    if (c->timed_last) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, c->ev0, c->ev1) == cudaSuccess) s.kernel_ms = ms;
        else cudaGetLastError();  // leave no stale error behind for the caller's next CUDA call
    }
    *stats = s;
    return BHK_OK;
}

bhk_status bhk_autotune(bhk_context* c, const bhk_frame_desc* frames, int32_t nframes, const bhk_trace_opts* opts,
                        bhk_trace_stats* chosen) {
    if (!c) return fail(BHK_EINVAL, "context is null");
    std::lock_guard<std::mutex> lock(c->mu);
    BHK_CUDA(cudaSetDevice(c->device));
    int64_t total = 0;
    bhk_status st = check_frames(frames, nframes, &total);
    if (st != BHK_OK) return st;
    st = ensure_outputs(c, static_cast<size_t>(total));
    if (st != BHK_OK) return st;
    bhk_trace_opts o{};
    if (opts) o = *opts;
    o.use_graph = 0;
    const int pi = o.precision == BHK_PREC_FP64 ? 0 : 1;
    const int blocks[] = {64, 128, 256};
    const int chunks[] = {32, 256};
    const int buckets[] = {1, 64, 512};
    const int budgets[] = {3, 1, 2};
    const bhk_rays_out out = own_outputs(c);
    float best = 1e30f;
    int bb = 128, bc = 32, bk = 1, br = 1;
    cudaEvent_t t0, t1;
    BHK_CUDA(cudaEventCreate(&t0));
    BHK_CUDA(cudaEventCreate(&t1));
    for (int rb : budgets)
    for (int blk : blocks)
        for (int ch : chunks)
            for (int bu : buckets) {
                const int rc = (pi == 0 || rb >= 3) ? 0 : rb;
                if (pi == 0 && rb != 3) continue;
                if (trace_blocks_per_sm(pi == 0, rc, blk) < 1) continue;
                o.block = blk;
                o.chunk = ch;
                o.sort_buckets = bu;
                o.reg_budget = rb;
                float t_best = 1e30f;
                for (int rep = 0; rep < 2; ++rep) {
                    BHK_CUDA(cudaEventRecord(t0, c->stream));
                    st = trace_frames_locked(c, frames, nframes, &o, &out, c->stream, false);
                    if (st != BHK_OK) {
                        cudaEventDestroy(t0);
                        cudaEventDestroy(t1);
                        return st;
                    }
                    BHK_CUDA(cudaEventRecord(t1, c->stream));
                    BHK_CUDA(cudaEventSynchronize(t1));
                    float ms = 0.0f;
                    BHK_CUDA(cudaEventElapsedTime(&ms, t0, t1));
                    t_best = std::min(t_best, ms);
                }
                if (t_best < best) {
                    best = t_best;
                    bb = blk; bc = ch; bk = bu; br = rb;
                }
            }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    c->tuned_block[pi] = bb;
    c->tuned_chunk[pi] = bc;
    c->tuned_buckets[pi] = bk;
    c->tuned_regcap[pi] = br;
    if (chosen) {
        *chosen = bhk_trace_stats{};
        chosen->block = bb;
        chosen->chunk = bc;
        chosen->sort_buckets = bk;
        chosen->reg_budget = br;
        chosen->kernel_ms = best;
        chosen->rays = total;
        o.block = bb; o.chunk = bc; o.sort_buckets = bk; o.reg_budget = br;
        chosen->grid = resolve(c, &o).grid;
    }
    return BHK_OK;
}

bhk_status bhk_critical_curve(double a, double r_obs, double theta_obs, int32_t samples, double* alpha, double* beta,
                              int32_t cap, int32_t* n) {
    if (!alpha || !beta || !n || cap < 0 || samples <= 0) return fail(BHK_EINVAL, "bad argument");
    const int m = (samples > 16 ? samples : 16) * 8 + 1;
    double* d_a = nullptr;
    double* d_b = nullptr;
    int* d_v = nullptr;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&d_a), sizeof(double) * m);
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&d_b), sizeof(double) * m);
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&d_v), sizeof(int) * m);
    std::vector<double> ha(m), hb(m);
    std::vector<int> hv(m);
    if (e == cudaSuccess) {
        launch_critical_curve(a, r_obs, theta_obs, samples, d_a, d_b, d_v, nullptr);
        e = cudaMemcpy(ha.data(), d_a, sizeof(double) * m, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(hb.data(), d_b, sizeof(double) * m, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(hv.data(), d_v, sizeof(int) * m, cudaMemcpyDeviceToHost);
    }
    if (d_a) cudaFree(d_a);
    if (d_b) cudaFree(d_b);
    if (d_v) cudaFree(d_v);
    if (e != cudaSuccess) return cuda_fail(e, "bhk_critical_curve");
    // Upper half along increasing orbit radius, then the mirrored lower half back.
    std::vector<int> idx;
    for (int k = 0; k < m; ++k)
        if (hv[k]) idx.push_back(k);
    int w = 0;
    for (size_t j = 0; j < idx.size() && w < cap; ++j, ++w) alpha[w] = ha[idx[j]], beta[w] = hb[idx[j]];
    for (size_t j = idx.size(); j-- > 0 && w < cap; ++w) alpha[w] = ha[idx[j]], beta[w] = -hb[idx[j]];
    *n = w;
    return BHK_OK;
}

}  // extern "C"
