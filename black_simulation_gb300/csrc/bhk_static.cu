// bhk_static.cu -- bhk_trace_frames_static: the batch tracer without any device allocation.
//
// Who needs it: callers that may not call cudaMalloc themselves or have the library call it on
// their behalf -- a host framework that owns the whole device-memory budget through its own pool
// and forbids side allocations, or a per-frame render loop where cudaMalloc/cudaFree would
// synchronise the device and stall the frame. This entry point takes the caller's output buffers
// and keeps every piece of working memory (launch records, queue counter, frame tetrads, rescue
// list) in one fixed array in the device image of libbhk, reserved when the library is loaded.
//
// Costs and limits of that choice:
//  - the array holds kStaticMaxRays rays and kStaticMaxFrames frames per call (6.1 MB), and
//    every GPU that loads libbhk keeps it until the process exits;
//  - all calls share the one array, whose contents persist from the previous call. The control
//    block (queue counter, statistics) and, with the cost sort, its bucket histogram are cleared at
//    the start of each call; everything else is rewritten before it is read. Calls that overlap on
//    the GPU (two streams, or two host threads without ordering between them) race on the array:
//    order them on one stream.
//  - the first call on a device looks up the array's device address (cudaGetSymbolAddress with
//    that device current) and caches it with the identity of the device's context; make that first
//    call before any stream capture. A call that finds a different context (after cudaDeviceReset)
//    looks the address up again, so it too belongs before any capture.
//  - the call is asynchronous and reports BHK_OK once its work is queued: rays that reach the step
//    cap show only as BHK_RAY_UNFINISHED in the outcome array (the context entry points synchronise
//    to return BHK_EUNFINISHED; this one never waits on the GPU).
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include <cuda.h>

#include "bhk_internal.h"

namespace bhk {
namespace {

constexpr int kStaticMaxRays = 65536;
constexpr int kStaticMaxFrames = 64;
constexpr int kStaticRescue = kStaticMaxRays / 4 + 1024;
constexpr int kMaxDevices = 64;

// Layout of the working memory inside the static array (offsets, 256-byte aligned).
struct Layout {
    size_t ctl, hist, offs, frames, geom, E, L, Q, vr, vth, gid, key, order, cf, vf, kf, khf, rescue, total;
};

constexpr size_t up256(size_t x) { return (x + 255) / 256 * 256; }

constexpr Layout make_layout() {
    Layout l{};
    size_t o = 0;
    l.ctl = o; o = up256(o + sizeof(Control));
    l.hist = o; o = up256(o + sizeof(unsigned) * kMaxBuckets);
    l.offs = o; o = up256(o + sizeof(unsigned) * kMaxBuckets);
    l.frames = o; o = up256(o + sizeof(FrameDev) * kStaticMaxFrames);
    l.geom = o; o = up256(o + sizeof(RayGeom) * kStaticMaxFrames);
    l.E = o; o = up256(o + sizeof(double) * kStaticMaxRays);
    l.L = o; o = up256(o + sizeof(double) * kStaticMaxRays);
    l.Q = o; o = up256(o + sizeof(double) * kStaticMaxRays);
    l.vr = o; o = up256(o + sizeof(double) * kStaticMaxRays);
    l.vth = o; o = up256(o + sizeof(double) * kStaticMaxRays);
    l.gid = o; o = up256(o + sizeof(int32_t) * kStaticMaxRays);
    l.key = o; o = up256(o + sizeof(uint16_t) * kStaticMaxRays);
    l.order = o; o = up256(o + sizeof(int32_t) * kStaticMaxRays);
    l.cf = o; o = up256(o + sizeof(float4) * kStaticMaxRays);
    l.vf = o; o = up256(o + sizeof(float2) * kStaticMaxRays);
    l.kf = o; o = up256(o + sizeof(float4) * kStaticMaxRays);
    l.khf = o; o = up256(o + sizeof(float2) * kStaticMaxRays);
    l.rescue = o; o = up256(o + sizeof(Rescue) * kStaticRescue);
    l.total = o;
    return l;
}

constexpr Layout kLayout = make_layout();

// The working memory of bhk_trace_frames_static, in the device image: no allocation at run time.
static __device__ __align__(256) unsigned char g_static_scratch[kLayout.total];

bhk_status fail(bhk_status s, const std::string& m) {
    set_last_error(m);
    return s;
}

// The frames' set-up (tetrads, lowered vectors, horizon, ISCO, capture and escape radii) is made on the
// host by the same code as bhk_trace_frames uses, so both entry points trace from identical bits, and
// travels to the device as kernel parameters: 64 x 408 + 8 bytes of frame records and 64 x 136 + 16
// bytes of geometries, each above the classic 4 KB limit and within the 32,764 bytes that CUDA 12.1 and
// later allow on Volta and later GPUs (this library is built by CUDA 13 for sm_103a only).
struct FrameTable {
    FrameDev f[kStaticMaxFrames];
    int n, pad;
};
struct GeomTable {
    RayGeom g[kStaticMaxFrames];
    long long n_rays;
    int n, pad;
};
static_assert(sizeof(FrameTable) <= 32764 && sizeof(GeomTable) <= 32764, "kernel parameter limit");

__global__ void stage_frames_kernel(FrameTable t, FrameDev* frames) {
    for (int i = threadIdx.x; i < t.n; i += blockDim.x) frames[i] = t.f[i];
}

__global__ void stage_geom_kernel(GeomTable t, RayGeom* geom, Control* ctl) {
    for (int i = threadIdx.x; i < t.n; i += blockDim.x) geom[i] = t.g[i];
    if (threadIdx.x == 0) ctl->n_rays = t.n_rays;
}

std::mutex g_addr_mu;
void* g_addr[kMaxDevices] = {};
unsigned long long g_ctx_id[kMaxDevices] = {};

// The two driver calls, taken through the runtime's entry-point query so that libbhk does not link
// libcuda directly (it loads on machines without a driver, where every call reports BHK_ECUDA).
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

bool driver_fns(CtxGetCurrentFn* cur, CtxGetIdFn* id) {
    static CtxGetCurrentFn f_cur = nullptr;
    static CtxGetIdFn f_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            f_cur = reinterpret_cast<CtxGetCurrentFn>(p);
        else
            cudaGetLastError();
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            f_id = reinterpret_cast<CtxGetIdFn>(p);
        else
            cudaGetLastError();
    });
    *cur = f_cur;
    *id = f_id;
    return f_cur && f_id;
}

// Unique id of the context the runtime uses on this thread for `device` (its primary context unless
// the caller made another current). cudaSetDevice binds the primary context where none is current,
// or after cudaDeviceReset destroyed the one that was.
bool current_context_id(int device, unsigned long long* id) {
    CtxGetCurrentFn get_cur;
    CtxGetIdFn get_id;
    if (!driver_fns(&get_cur, &get_id)) return false;
    CUcontext cur = nullptr;
    if (get_cur(&cur) == CUDA_SUCCESS && cur && get_id(cur, id) == CUDA_SUCCESS) return true;
    if (cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    cur = nullptr;
    return get_cur(&cur) == CUDA_SUCCESS && cur && get_id(cur, id) == CUDA_SUCCESS;
}

// Device address of the static array on the current device: looked up (cudaGetSymbolAddress) once per
// device and context, with that device current.
bhk_status scratch_address(int device, unsigned char** out) {
    unsigned long long id = 0;
    if (!current_context_id(device, &id)) return fail(BHK_ECUDA, "no current CUDA context for the device");
    std::lock_guard<std::mutex> lock(g_addr_mu);
    if (!g_addr[device] || g_ctx_id[device] != id) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(BHK_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        }
        g_addr[device] = p;
        g_ctx_id[device] = id;
    }
    *out = static_cast<unsigned char*>(g_addr[device]);
    return BHK_OK;
}

}  // namespace
}  // namespace bhk

using namespace bhk;

extern "C" bhk_status bhk_trace_frames_static(const bhk_frame_desc* frames, int32_t nframes,
                                              const bhk_trace_opts* opts, const bhk_rays_out* out, void* stream) {
    if (!frames || nframes <= 0 || !out) return fail(BHK_EINVAL, "frames, nframes and out are required");
    if (nframes > kStaticMaxFrames)
        return fail(BHK_EINVAL, "bhk_trace_frames_static takes at most 64 frames per call");
    // The same frame checks as bhk_trace_frames (naked singularities included), then the array's limits.
    int64_t total = 0;
    const bhk_status vs = validate_frames(frames, nframes, &total);
    if (vs != BHK_OK) return vs;
    if (total > kStaticMaxRays)
        return fail(BHK_EINVAL, "bhk_trace_frames_static takes at most 65536 rays per call (the static scratch)");
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kMaxDevices)
        return fail(BHK_ECUDA, "no usable CUDA device");
    unsigned char* base = nullptr;
    bhk_status st = scratch_address(device, &base);
    if (st != BHK_OK) return st;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);

    bhk_trace_opts d{};
    const bhk_trace_opts& o = opts ? *opts : d;
    TraceParams p{};
    const bool fp64 = o.precision == BHK_PREC_FP64;
    p.rtol = o.rtol > 0.0 ? o.rtol : (fp64 ? 1e-10 : 1e-6);
    p.eps = o.capture_eps > 0.0 ? o.capture_eps : 1e-6;
    p.r_escape = o.r_escape > 0.0 ? o.r_escape : 1000.0;
    p.max_steps = o.max_steps > 0 ? o.max_steps : 20000;
    p.reproject_every = o.reproject_every > 0 ? o.reproject_every : 0;
    p.tol0 = std::fmin(std::fmax(std::pow(p.rtol, 0.2), 1e-3), 0.05);
    p.rtol_f = static_cast<float>(p.rtol);
    p.tol0_f = static_cast<float>(p.tol0);
    p.pole_frac = o.pole_step_frac > 0.0 ? static_cast<float>(o.pole_step_frac)
                  : (o.pole_step_frac < 0.0 ? 0.0f
                     : static_cast<float>(std::fmin(0.5, 0.1 * std::pow(p.rtol / 1e-6, 0.2))));
    p.fp64_turning = (!fp64 && o.fp64_turning) ? 1 : 0;
    int block = o.block > 0 ? std::min(o.block, 256) : 128;
    p.chunk = ((o.chunk > 32 ? o.chunk : 32) + 31) / 32 * 32;  // whole batches of 32 (one per lane)
    p.buckets = std::min(o.sort_buckets > 0 ? o.sort_buckets : 1, kMaxBuckets);
    const int rb = o.reg_budget > 0 ? o.reg_budget : 1;
    const int regcap = p.fp64_turning ? 1 : ((fp64 || rb >= 3) ? 0 : rb);
    if (regcap > 0) block = std::min(block, 128);
    const int grid = std::max(1, trace_blocks_per_sm(fp64, regcap, block)) * sms;

    Control* ctl = reinterpret_cast<Control*>(base + kLayout.ctl);
    FrameDev* fdev = reinterpret_cast<FrameDev*>(base + kLayout.frames);
    RayGeom* geom = reinterpret_cast<RayGeom*>(base + kLayout.geom);
    LaunchSoA L{reinterpret_cast<double*>(base + kLayout.E), reinterpret_cast<double*>(base + kLayout.L),
                reinterpret_cast<double*>(base + kLayout.Q), reinterpret_cast<double*>(base + kLayout.vr),
                reinterpret_cast<double*>(base + kLayout.vth), reinterpret_cast<int32_t*>(base + kLayout.gid),
                reinterpret_cast<uint16_t*>(base + kLayout.key), reinterpret_cast<float4*>(base + kLayout.cf),
                reinterpret_cast<float2*>(base + kLayout.vf),
                fp64 ? nullptr : reinterpret_cast<float4*>(base + kLayout.kf),
                fp64 ? nullptr : reinterpret_cast<float2*>(base + kLayout.khf)};
    SortScratch S{reinterpret_cast<unsigned*>(base + kLayout.hist), reinterpret_cast<unsigned*>(base + kLayout.offs),
                  reinterpret_cast<int32_t*>(base + kLayout.order)};
    Rescue* rescue = reinterpret_cast<Rescue*>(base + kLayout.rescue);
    Outputs outs{out->outcome, out->r_disk,   out->phi_disk, out->g, out->theta_inf, out->phi_inf, out->steps,
                 out->rejected, out->energy, out->g_camera, out->b,        out->q, out->r_min,     out->delay,
                 out->turns};

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // Host-side tables (about 35 KB on this thread's stack; no allocation).
    FrameTable ft;
    GeomTable gt;
    std::memset(static_cast<void*>(&ft), 0, sizeof(ft));
    std::memset(static_cast<void*>(&gt), 0, sizeof(gt));
    for (int i = 0; i < nframes; ++i) ft.f[i].d = frames[i];
    gt.n_rays = setup_frames_host(ft.f, gt.g, nframes, p);
    ft.n = gt.n = nframes;
    cudaError_t e = cudaMemsetAsync(ctl, 0, sizeof(Control), s);
    if (e == cudaSuccess && p.buckets > 1) e = cudaMemsetAsync(S.hist, 0, sizeof(unsigned) * kMaxBuckets, s);
    if (e != cudaSuccess) return fail(BHK_ECUDA, std::string("clearing the control block: ") + cudaGetErrorString(e));
    stage_frames_kernel<<<1, 64, 0, s>>>(ft, fdev);
    stage_geom_kernel<<<1, 64, 0, s>>>(gt, geom, ctl);
    launch_rays_frames(fdev, geom, nframes, L, p, ctl, sms * 8, s);
    const int32_t* order = nullptr;
    if (p.buckets > 1) {
        launch_sort(L, S, p, ctl, sms * 8, s);
        order = S.order;
    }
    launch_trace(fp64, regcap, L, geom, order, outs, rescue, kStaticRescue, p, ctl, block, grid, s);
    if (!fp64) launch_rescue(L, geom, outs, rescue, kStaticRescue, p, ctl, sms, s);
    launch_constants_out(L, outs, ctl, sms * 8, s);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(BHK_ECUDA, std::string("launch: ") + cudaGetErrorString(e));
    return BHK_OK;
}
