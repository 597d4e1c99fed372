// bhk_surrogate.cu -- the learned part: a BF16 MLP surrogate of the tracer, trained and run by
// hand-written tcgen05 kernels (FP32 accumulation in TMEM, FP32 master weights and Adam state).
//
// Network (per ray): inputs (a, theta_obs, log10 r_obs, alpha, beta) -> normalised to [-1, 1]^5 ->
// 64 Fourier features [sin, cos](2 pi B u) with a fixed seeded B (32 x 5) -> 4 x (256, SiLU) ->
// head of 8 (3 outcome logits, r_disk / 30, log g, unit escape vector), padded to 16 for the MMA.
//
// Every GEMM is C = A * B^T with BF16 operands in global memory, row-major:
//   forward   Y   = X * W^T         A = activations [rows x K] (K-major),  B = W [N x K] (K-major)
//   backward  dX  = dY * W          A = dY [rows x N] (K-major),           B = W^T stored [K x N] (K-major)
//             dW  = dY^T * X        A = dY [rows x N] read MN-major,       B = X [rows x K] read MN-major
//                                   (split over rows; the head's dY^T, 16 rows, is stored K-major)
// so the activations and gradients exist in one layout only.
//
// GEMM kernel: one CTA computes a 128 x BN tile; TMA brings 64-wide K chunks of A and B into a ring
// of shared-memory stages (128-byte swizzle); one thread issues tcgen05.mma (M = 128, N = BN, K = 16
// per instruction) into a TMEM accumulator and commits each stage back to the producer; after the
// last chunk eight warps read the accumulator with tcgen05.ld (warps w and w + 4 own rows 32w..32w+31)
// and run the epilogue: the hidden layers' through shared-memory boxes and TMA tensor stores. Every
// wait is bounded; a timeout sets an error flag the host checks.
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "bhk_device.cuh"
#include "bhk_internal.h"
#include "bhk_tc.cuh"

namespace bhk {
namespace sur {

using bf16 = __nv_bfloat16;

// The network's shape: 5 inputs, 32 Fourier frequencies (64 features), 8 outputs padded to 16 for the
// MMA, 5 layers.
constexpr int kIn = 5, kFreq = 32, kFeat = 64, kOut = 8, kOutPad = 16, kLayers = 5;
constexpr int kTileM = 128;
constexpr int kChunkK = 64;
constexpr int kABytes = kTileM * kChunkK * 2;  // 16 KB

enum Epi : int { kStoreF32 = 0, kBiasSilu = 1, kDsilu = 2, kAtomicF32 = 3, kReduceF32 = 5, kHeadLoss = 6 };

struct EpiArgs {
    int M, N;              // logical output extent (rows, columns)
    const float* bias;     // [N] or null
    float* f32;            // kStoreF32 / kAtomicF32 output, row-major with ld_f32
    int ld_f32;
    float* colsum;         // kDsilu: column sums of the output (bias gradient), atomically
    int no_store;          // kDsilu in layer_kernel: dZ is not written (only the fused gradients are used)
    int wg;                // layer_kernel<kDsilu, 256>: the fused weight gradient's width, 64 or 256 (0: 256)
    int late_weights;      // layer_kernel: the weights and biases were written by the kernel launched just
                           // before (the optimiser step): load them after the programmatic-launch wait
    int early_a;           // layer_kernel (forward): A was written at least two launches upstream, so the
                           // first ring's worth of its chunks may be loaded before that wait
    // kHeadLoss (the head's forward with the loss fused in; colsum takes the head's bias gradient):
    const uint8_t* cls;    // per row: target class 1 captured, 2 disk, 3 escaped
    const float* tgt;      // per row: 8 targets
    bf16* dy_rm;           // dLoss/dY, row-major [M x 16], and transposed [16 x ld_t]
    bf16* dy_t;
    int ld_t;
    float* loss;           // the four loss terms, atomically
    float inv_n;
    float4 lw;             // loss weights (CE, r_disk, ln g, direction)
};

// Loss of one row (y: the head's 16 outputs, c: target class - 1, tg: its 8 targets) and its gradient d
// with respect to y, scaled by inv_n; terms = (cross-entropy, r_disk, ln g, direction) unweighted:
//   cross-entropy over the 3 outcome logits; disk rays: squared error of r_disk / 30 and of log g;
//   escaped rays: squared error of the 3-vector escape direction. The gradient is that of the weighted
//   sum w.x CE + w.y MSE(r) + w.z MSE(ln g) + w.w MSE(dir).
__device__ __forceinline__ void row_loss(const float (&y)[kOutPad], int c, const float* __restrict__ tg, float inv_n,
                                         float4 w, float (&d)[kOutPad], float (&terms)[4]) {
#pragma unroll
    for (int i = 0; i < kOutPad; ++i) d[i] = 0.0f;
    terms[0] = terms[1] = terms[2] = terms[3] = 0.0f;
    const float mx = fmaxf(y[0], fmaxf(y[1], y[2]));
    const float e0 = __expf(y[0] - mx), e1 = __expf(y[1] - mx), e2 = __expf(y[2] - mx);
    const float z = e0 + e1 + e2;
    const float p[3] = {e0 / z, e1 / z, e2 / z};
    if (c >= 0 && c < 3) {
        terms[0] = -__logf(fmaxf(p[c], 1e-30f));
        for (int k = 0; k < 3; ++k) d[k] = w.x * (p[k] - (k == c ? 1.0f : 0.0f)) * inv_n;
    }
    if (c == 1) {  // disk
        const float er = y[3] - tg[3], eg = y[4] - tg[4];
        terms[1] = er * er;
        terms[2] = eg * eg;
        d[3] = w.y * 2.0f * er * inv_n;
        d[4] = w.z * 2.0f * eg * inv_n;
    } else if (c == 2) {  // escaped
        for (int k = 5; k < 8; ++k) {
            const float ev = y[k] - tg[k];
            terms[3] += ev * ev;
            d[k] = w.w * 2.0f * ev * inv_n;
        }
    }
}

// Pipeline depth: the network's GEMMs have K <= 256 (4 chunks) and run two CTAs (each 256 TMEM
// columns at most) per SM, so that one CTA's epilogue overlaps the other's main loop. The training
// head (kHeadLoss, 16 wide, one 128-row tile per CTA) keeps two stages, so that four CTAs fit an SM and
// the whole batch runs in one wave. The split-K
// weight gradients stream long K ranges (~14 chunks a CTA) with a light epilogue: one CTA per SM with
// a deep ring, so that the TMA latency of the next chunks hides behind the current MMAs.
template <int BN, int EPI>
__host__ __device__ constexpr int gemm_stages() {
    return EPI == kReduceF32 ? (BN >= 256 ? 4 : 8) : EPI == kHeadLoss ? 2 : (BN >= 256 ? 2 : 4);
}

template <int BN, int EPI>
__host__ __device__ constexpr int gemm_smem_bytes() {
    return gemm_stages<BN, EPI>() * (kABytes + BN * kChunkK * 2) + 1024 + 256 + BN * 4;
}

// Logistic sigmoid as 1/2 + tanh(z/2)/2 on the hardware tanh (one MUFU operation; relative error of
// tanh.approx.f32 about 2^-11). Training and inference use this same SiLU.
__device__ __forceinline__ float sigmoidf(float z) {
    float t;
    asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(0.5f * z));
    return fmaf(0.5f, t, 0.5f);
}

// The network's activation: SiLU of two pre-activations passed as halves h = z / 2 (FP32),
// silu(z) = h + h tanh(h), evaluated in BF16x2 -- h rounded to BF16, the hardware BF16x2 tanh, one
// fused multiply-add rounded to BF16 -- and returned packed (element 0 in the low half). One MUFU
// operation per two activations; training and inference both use exactly this.
__device__ __forceinline__ uint32_t silu2_half(float h0, float h1) {
    uint32_t hb, t, a;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(hb) : "f"(h1), "f"(h0));
    asm("tanh.approx.bf16x2 %0, %1;" : "=r"(t) : "r"(hb));
    asm("fma.rn.bf16x2 %0, %1, %2, %1;" : "=r"(a) : "r"(hb), "r"(t));
    return a;
}

// Sums each of 16 per-lane values over the warp's 32 lanes by recursive halving (16 shuffles). The
// total of column `col` (= bits 4..1 of the lane) is returned in lanes 2 col and 2 col + 1.
__device__ __forceinline__ float warp_colsum16(const float (&x)[16], int lane, int& col) {
    const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4, b1 = lane & 2;
    float y[8], z[4], w[2];
#pragma unroll
    for (int i = 0; i < 8; ++i) y[i] = (b4 ? x[8 + i] : x[i]) + __shfl_xor_sync(0xffffffffu, b4 ? x[i] : x[8 + i], 16);
#pragma unroll
    for (int i = 0; i < 4; ++i) z[i] = (b3 ? y[4 + i] : y[i]) + __shfl_xor_sync(0xffffffffu, b3 ? y[i] : y[4 + i], 8);
#pragma unroll
    for (int i = 0; i < 2; ++i) w[i] = (b2 ? z[2 + i] : z[i]) + __shfl_xor_sync(0xffffffffu, b2 ? z[i] : z[2 + i], 4);
    float v = (b1 ? w[1] : w[0]) + __shfl_xor_sync(0xffffffffu, b1 ? w[0] : w[1], 2);
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    col = (b4 ? 8 : 0) + (b3 ? 4 : 0) + (b2 ? 2 : 0) + (b1 ? 1 : 0);
    return v;
}

// Threads of a GEMM CTA: thread 0 loads and issues; in the epilogue, warps w and w + 4 read TMEM lane
// quadrant w and split the tile's columns (BN >= 32; a 16-wide tile uses warps 0-3 alone).
constexpr int kGemmThreads = 256;

// Shared memory a warp of the staged epilogue uses (two 4 KB TMA boxes), carved from the idle ring.
constexpr int kWarpStage = 8192;

// Split-K weight-gradient epilogue (kReduceF32): the tile's FP32 partial product goes straight into the
// FP32 gradient through TMA reductions (element-wise adds performed in L2) -- no workspace and no
// reduction pass; the order in which the splits' adds land is not fixed. Warp (quad, part) owns the 32
// rows of TMEM lane quadrant `quad` and BN / 2 columns: per 32 columns one tcgen05.ld, one [32 x 32] FP32
// box written into shared memory under the 128-byte swizzle (double-buffered per warp) and one TMA
// reduction. Rows at or past M are skipped a whole box at a time (TMA clips partial boxes).
template <int BN>
__device__ __forceinline__ void epilogue_reduce(const CUtensorMap* tmG, const EpiArgs& ea, uint32_t tmem,
                                                uint8_t* stage_base, int m0, int n0) {
    static_assert(BN % 64 == 0, "two warps of 32-column boxes per lane quadrant");
    constexpr int kColsW = BN / 2;  // columns per warp
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int quad = warp & 3, part = warp >> 2;
    const int y0 = m0 + 32 * quad;
    if (y0 >= ea.M) return;
    uint8_t* wb = stage_base + warp * kWarpStage;
    const uint32_t trow = tmem + (static_cast<uint32_t>(32 * quad) << 16) + part * kColsW;
    const int sw = lane & 7;
#pragma unroll 1
    for (int j = 0; j < kColsW / 32; ++j) {
        uint32_t r[32];
        tc::tmem_ld32_issue(trow + 32 * j, r);
        tc::tmem_wait32(r);
        uint8_t* box = wb + (j & 1) * 4096;
        if (j >= 2) {  // the reduction of box j - 2 has read this buffer
            if (lane == 0) tc::bulk_wait_read_but_one();
            __syncwarp();
        }
        uint4* row = reinterpret_cast<uint4*>(box + lane * 128);
#pragma unroll
        for (int c = 0; c < 8; ++c) row[c ^ sw] = make_uint4(r[4 * c], r[4 * c + 1], r[4 * c + 2], r[4 * c + 3]);
        tc::fence_proxy_async();
        __syncwarp();
        if (lane == 0) {
            tc::tma_reduce_add_2d(tmG, box, n0 + part * kColsW + 32 * j, y0);
            tc::bulk_commit();
        }
    }
    if (lane == 0) tc::bulk_wait_all();
    __syncwarp();
}

// Staged epilogue of the hidden layers (kBiasSilu: Z = acc + b and A = silu(Z); kDsilu: dZ = acc *
// silu'(Z) and the bias gradient). Warp (quad, part) owns the 32 rows of TMEM lane quadrant `quad` and
// kBoxes 64-column boxes of the tile. Each box's outputs are written into shared memory in the layout of
// a TMA box -- row-major [32 rows][64 columns] under the 128-byte swizzle (the 16-byte chunk c of row r at
// chunk c ^ (r & 7)) -- and leave with one TMA tensor store per output, so a warp issues a few bulk
// stores per box instead of 32-row scattered vector stores. kDsilu reads Z the same way: TMA loads of
// the warp's boxes, dZ written over them in place. sx holds the tile's bias (kBiasSilu) or its column
// sums (kDsilu). Returns false if a wait for the Z loads timed out.
template <int BN, int EPI>
__device__ __forceinline__ bool epilogue_staged(const CUtensorMap* tmZ, const CUtensorMap* tmR, const EpiArgs& ea,
                                                uint32_t tmem, uint8_t* stage_base, float* sx, uint64_t* zbar, int m0,
                                                int n0) {
    static_assert(BN % 64 == 0, "the staged epilogue works on 64-column boxes");
    constexpr int kSplitS = BN >= 128 ? 2 : 1;   // warps sharing a lane quadrant
    constexpr int kBoxes = BN / (64 * kSplitS);  // boxes per warp
    constexpr int kG = 4 * kBoxes;               // 16-column groups per warp
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int quad = warp & 3, part = warp >> 2;
    if constexpr (EPI == kBiasSilu) {
        for (int i = threadIdx.x; i < BN; i += blockDim.x) sx[i] = n0 + i < ea.N ? ea.bias[n0 + i] : 0.0f;
    } else {
        for (int i = threadIdx.x; i < BN; i += blockDim.x) sx[i] = 0.0f;
    }
    __syncthreads();
    bool ok = true;
    if (part < kSplitS) {
        uint8_t* wb = stage_base + warp * kWarpStage;
        const int y0 = m0 + 32 * quad;
        const bool live = y0 + lane < ea.M;
        const int c_lo = part * kBoxes * 64;  // the warp's first tile column
        if constexpr (EPI == kDsilu) {
            if (lane == 0) {
                tc::mbar_expect_tx(&zbar[warp], kBoxes * 4096);
                for (int b = 0; b < kBoxes; ++b) tc::tma_load_2d(wb + b * 4096, tmZ, n0 + c_lo + 64 * b, y0, &zbar[warp]);
            }
        }
        const uint32_t trow = tmem + (static_cast<uint32_t>(32 * quad) << 16);
        const int sw = lane & 7;
        auto process = [&](int gi, const uint32_t (&r)[16]) {
            const int b = gi >> 2, g = gi & 3, cb = c_lo + 16 * gi;
            if constexpr (EPI == kBiasSilu) {
                if (g == 0 && b > 0) {  // the previous box's stores must have read the staging it reuses
                    if (lane == 0) tc::bulk_wait_read_all();
                    __syncwarp();
                }
            }
            __align__(16) bf16 ob[16];
            if constexpr (EPI == kBiasSilu) {
                __align__(16) bf16 zb[16];
#pragma unroll
                for (int i = 0; i < 16; i += 2) {
                    const float z0 = __uint_as_float(r[i]) + sx[cb + i], z1 = __uint_as_float(r[i + 1]) + sx[cb + i + 1];
                    zb[i] = __float2bfloat16_rn(z0);
                    zb[i + 1] = __float2bfloat16_rn(z1);
                    *reinterpret_cast<uint32_t*>(&ob[i]) = silu2_half(0.5f * z0, 0.5f * z1);
                }
                uint4* zrow = reinterpret_cast<uint4*>(wb + lane * 128);
                uint4* arow = reinterpret_cast<uint4*>(wb + 4096 + lane * 128);
                zrow[(2 * g) ^ sw] = reinterpret_cast<const uint4*>(zb)[0];
                zrow[(2 * g + 1) ^ sw] = reinterpret_cast<const uint4*>(zb)[1];
                arow[(2 * g) ^ sw] = reinterpret_cast<const uint4*>(ob)[0];
                arow[(2 * g + 1) ^ sw] = reinterpret_cast<const uint4*>(ob)[1];
            } else {
                uint4* zrow = reinterpret_cast<uint4*>(wb + b * 4096 + lane * 128);
                __align__(16) bf16 zin[16];
                reinterpret_cast<uint4*>(zin)[0] = zrow[(2 * g) ^ sw];
                reinterpret_cast<uint4*>(zin)[1] = zrow[(2 * g + 1) ^ sw];
                float dz[16];
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    const float z = __bfloat162float(zin[i]);
                    const float sg = sigmoidf(z);
                    dz[i] = live ? __uint_as_float(r[i]) * sg * (1.0f + z * (1.0f - sg)) : 0.0f;
                    ob[i] = __float2bfloat16_rn(dz[i]);
                }
                zrow[(2 * g) ^ sw] = reinterpret_cast<const uint4*>(ob)[0];
                zrow[(2 * g + 1) ^ sw] = reinterpret_cast<const uint4*>(ob)[1];
                if (ea.colsum) {
                    int col;
                    const float tot = warp_colsum16(dz, lane, col);
                    if (!(lane & 1)) atomicAdd(&sx[cb + col], tot);
                }
            }
            if (g == 3) {  // the box is complete: hand it to the TMA unit
                tc::fence_proxy_async();
                __syncwarp();
                if (lane == 0) {
                    const int x = n0 + c_lo + 64 * b;
                    if constexpr (EPI == kBiasSilu) {
                        tc::tma_store_2d(tmZ, wb, x, y0);
                        tc::tma_store_2d(tmR, wb + 4096, x, y0);
                    } else {
                        tc::tma_store_2d(tmR, wb + b * 4096, x, y0);
                    }
                    tc::bulk_commit();
                }
            }
        };
        uint32_t ra[16], rb[16];
        tc::tmem_ld16_issue(trow + c_lo, ra);
        if constexpr (EPI == kDsilu) {
            ok = __all_sync(0xffffffffu, tc::mbar_wait(&zbar[warp], 0) ? 1 : 0) != 0;
            // A timed-out wait: give the loads in flight a second bounded wait before the CTA exits.
            if (!ok) tc::mbar_wait(&zbar[warp], 0);
        }
        tc::tmem_wait16(ra);
        if (ok) {
#pragma unroll 1
            for (int gi = 0; gi < kG; gi += 2) {
                tc::tmem_ld16_issue(trow + c_lo + 16 * (gi + 1), rb);
                process(gi, ra);
                tc::tmem_wait16(rb);
                if (gi + 2 < kG) tc::tmem_ld16_issue(trow + c_lo + 16 * (gi + 2), ra);
                process(gi + 1, rb);
                if (gi + 2 < kG) tc::tmem_wait16(ra);
            }
        }
        if (lane == 0) tc::bulk_wait_all();
        __syncwarp();
    }
    if constexpr (EPI == kDsilu) {
        __syncthreads();
        if (ea.colsum)
            for (int i = threadIdx.x; i < BN && n0 + i < ea.N; i += blockDim.x) atomicAdd(&ea.colsum[n0 + i], sx[i]);
    }
    return ok;
}

// MAJ bit 0: A is MN-major (a row-major [K x M] matrix, loaded as 64 x 64 boxes, two per 128-row tile);
// bit 1: B is MN-major ([K x N], BN / 64 boxes). Otherwise the operand is K-major ([M x K], [N x K]).
template <int BN, int EPI, int MAJ = 0>
__global__ void __launch_bounds__(kGemmThreads, 2)
gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
            const __grid_constant__ CUtensorMap tmZ, const __grid_constant__ CUtensorMap tmR, EpiArgs ea, int K,
            int k_per_split, int* err) {
    constexpr int kStages = gemm_stages<BN, EPI>();
    constexpr int kBBytes = BN * kChunkK * 2;
    constexpr uint32_t kCols = BN < 32 ? 32 : BN;
    constexpr bool kAmn = (MAJ & 1) != 0, kBmn = (MAJ & 2) != 0;
    static_assert(!kBmn || BN % 64 == 0, "an MN-major B tile is made of 64-wide boxes");
    constexpr uint32_t kIdesc = tc::idesc_bf16(kTileM, BN, kAmn, kBmn);
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t* sA = smem;
    uint8_t* sB = smem + kStages * kABytes;
    uint64_t* full = reinterpret_cast<uint64_t*>(sB + kStages * kBBytes);
    uint64_t* empty = full + kStages;
    uint64_t* accbar = empty + kStages;
    uint64_t* zbar = accbar + 1;  // one per warp: the staged epilogue's Z loads (kDsilu)
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(zbar + kGemmThreads / 32);
    int* fail = reinterpret_cast<int*>(tmem_slot + 1);
    float* sx = reinterpret_cast<float*>(full) + 64;  // past the barriers (<= 256 bytes): BN floats

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * kTileM, n0 = blockIdx.y * BN;
    const int k_begin = blockIdx.z * k_per_split;
    const int k_end = min(K, k_begin + k_per_split);
    const int nchunks = k_end > k_begin ? (k_end - k_begin + kChunkK - 1) / kChunkK : 0;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        tc::mbar_init(accbar, 1);
        for (int w = 0; w < kGemmThreads / 32; ++w) tc::mbar_init(&zbar[w], 1);
        *fail = 0;
        tc::fence_mbar_init();
        tc::prefetch_tmap(&tmA);
        tc::prefetch_tmap(&tmB);
    }
    if (warp == 0) tc::tmem_alloc(tmem_slot, kCols);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    // Launched programmatically: the previous grid of the stream has finished before any global access.
    tc::grid_dep_wait();
    tc::grid_dep_launch();

    if (threadIdx.x == 0) {
        auto load = [&](int stage, int chunk) {
            tc::mbar_expect_tx(&full[stage], kABytes + kBBytes);
            const int kx = k_begin + chunk * kChunkK;
            if constexpr (kAmn) {
                tc::tma_load_2d(sA + stage * kABytes, &tmA, m0, kx, &full[stage]);
                tc::tma_load_2d(sA + stage * kABytes + kABytes / 2, &tmA, m0 + 64, kx, &full[stage]);
            } else {
                tc::tma_load_2d(sA + stage * kABytes, &tmA, kx, m0, &full[stage]);
            }
            if constexpr (kBmn) {
#pragma unroll
                for (int j = 0; j < BN / 64; ++j)
                    tc::tma_load_2d(sB + stage * kBBytes + j * 8192, &tmB, n0 + 64 * j, kx, &full[stage]);
            } else {
                tc::tma_load_2d(sB + stage * kBBytes, &tmB, kx, n0, &full[stage]);
            }
        };
        bool ok = true;
        int loaded = 0;
        for (; loaded < nchunks && loaded < kStages; ++loaded) load(loaded, loaded);
        int c = 0;
        for (; c < nchunks; ++c) {
            const int s = c % kStages;
            if (!tc::mbar_wait(&full[s], (c / kStages) & 1)) {
                ok = false;
                break;
            }
            tc::fence_after_sync();
            // A K = 16 slice: +32 bytes inside the atom (K-major), +2048 bytes (MN-major: two 8-row atoms).
            const uint64_t ad = kAmn ? tc::smem_desc_sw128_mn(sA + s * kABytes, kABytes / 2)
                                     : tc::smem_desc_sw128(sA + s * kABytes);
            const uint64_t bd = kBmn ? tc::smem_desc_sw128_mn(sB + s * kBBytes, 8192) : tc::smem_desc_sw128(sB + s * kBBytes);
            constexpr uint64_t kStepA = kAmn ? 2048 >> 4 : 2, kStepB = kBmn ? 2048 >> 4 : 2;
#pragma unroll
            for (int kk = 0; kk < kChunkK / 16; ++kk)
                tc::mma_bf16(tmem, ad + kStepA * kk, bd + kStepB * kk, kIdesc, (c > 0 || kk > 0) ? 1u : 0u);
            tc::mma_commit(&empty[s]);
            // Refill the stage of the previous chunk once its MMAs are done (they run in order).
            if (c >= 1 && loaded < nchunks) {
                const int pc = c - 1, ps = pc % kStages;
                if (!tc::mbar_wait(&empty[ps], (pc / kStages) & 1)) {
                    ok = false;
                    ++c;
                    break;
                }
                load(ps, loaded);
                ++loaded;
            }
        }
        tc::mma_commit(accbar);
        if (!ok) {
            *fail = 1;
            atomicExch(err, 1);
            // Let the loads already in flight land before the CTA exits (bounded).
            for (int q = c; q < loaded; ++q) tc::mbar_wait(&full[q % kStages], (q / kStages) & 1);
        }
    }
    // The decision to run the epilogue is taken by the whole CTA (it contains block barriers).
    const int acc_ready = __syncthreads_and(tc::mbar_wait(accbar, 0) ? 1 : 0);
    tc::fence_after_sync();
    if (!acc_ready && threadIdx.x == 0) atomicExch(err, 1);
    if (acc_ready && !*fail && nchunks > 0) {
        if constexpr (EPI == kBiasSilu || EPI == kDsilu) {
            // The pipeline's shared memory is idle now: it holds the warps' output boxes.
            if (!epilogue_staged<BN, EPI>(&tmZ, &tmR, ea, tmem, sA, sx, zbar, m0, n0)) atomicExch(err, 1);
        } else if constexpr (EPI == kReduceF32) {
            epilogue_reduce<BN>(&tmZ, ea, tmem, sA, m0, n0);
        } else if constexpr (EPI == kHeadLoss) {
            // The head (BN = 16: warps 0-3, lane = row) with the loss: Y = acc + b, then the row's loss
            // terms and dLoss/dY (BF16, both layouts); the bias gradient and the loss terms summed over the
            // CTA's rows (shuffles, then the four warps through the idle ring) and added atomically.
            static_assert(BN == 16, "the head is 16 wide");
            float d[kOutPad], terms[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
            for (int i = 0; i < kOutPad; ++i) d[i] = 0.0f;
            if (warp < 4) {
                const int m = m0 + 32 * warp + lane;
                uint32_t r[16];
                tc::tmem_ld16_issue(tmem + (static_cast<uint32_t>(32 * warp) << 16), r);
                tc::tmem_wait16(r);
                if (m < ea.M) {
                    float y[kOutPad];
#pragma unroll
                    for (int i = 0; i < kOutPad; ++i) y[i] = __uint_as_float(r[i]) + ea.bias[i];
                    row_loss(y, static_cast<int>(ea.cls[m]) - 1, ea.tgt + static_cast<size_t>(m) * kOut, ea.inv_n,
                             ea.lw, d, terms);
                    __align__(16) bf16 ob[kOutPad];
#pragma unroll
                    for (int i = 0; i < kOutPad; ++i) ob[i] = __float2bfloat16_rn(d[i]);
                    uint4* dst = reinterpret_cast<uint4*>(ea.dy_rm + static_cast<size_t>(m) * kOutPad);
                    dst[0] = reinterpret_cast<const uint4*>(ob)[0];
                    dst[1] = reinterpret_cast<const uint4*>(ob)[1];
#pragma unroll
                    for (int i = 0; i < kOutPad; ++i) ea.dy_t[static_cast<size_t>(i) * ea.ld_t + m] = ob[i];
                }
            }
            float* red = reinterpret_cast<float*>(sA);
            if (warp < 4) {
#pragma unroll
                for (int i = 0; i < kOutPad + 4; ++i) {
                    float v = i < kOutPad ? d[i] : terms[i - kOutPad] * ea.inv_n;
                    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
                    if (lane == 0) red[warp * (kOutPad + 4) + i] = v;
                }
            }
            __syncthreads();
            if (threadIdx.x < kOutPad + 4) {
                float v = 0.0f;
                for (int q = 0; q < 4; ++q) v += red[q * (kOutPad + 4) + threadIdx.x];
                if (threadIdx.x < kOutPad) {
                    if (v != 0.0f) atomicAdd(&ea.colsum[threadIdx.x], v);
                } else {
                    atomicAdd(&ea.loss[threadIdx.x - kOutPad], v);
                }
            }
        } else {
            constexpr int kJ = BN / 16;                  // 16-column groups of the tile
            constexpr int kSplit = kJ >= 2 ? 2 : 1;      // warps sharing a lane quadrant
            const int quad = warp & 3, part = warp >> 2; // TMEM lane quadrant, share of the columns
            const int j_lo = part * kJ / kSplit, j_hi = (part + 1) * kJ / kSplit;
            const int row = 32 * quad + lane;
            const int m = m0 + row;
            const bool live = m < ea.M;
            // The accumulator is read 16 columns at a time, the next load in flight while the current
            // columns are processed.
            const uint32_t trow = tmem + (static_cast<uint32_t>(32 * quad) << 16);
            auto process = [&](int j, const uint32_t (&r)[16]) {
                float v[16];
#pragma unroll
                for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
                const int nb = n0 + 16 * j;
                if (nb >= ea.N || !live) return;
                if constexpr (EPI == kStoreF32) {
                    for (int i = 0; i < 16; ++i)
                        if (nb + i < ea.N)
                            ea.f32[static_cast<size_t>(m) * ea.ld_f32 + nb + i] = v[i] + (ea.bias ? ea.bias[nb + i] : 0.0f);
                } else {  // kAtomicF32
                    for (int i = 0; i < 16; ++i)
                        if (nb + i < ea.N) atomicAdd(&ea.f32[static_cast<size_t>(m) * ea.ld_f32 + nb + i], v[i]);
                }
            };
            // Warps without columns (a 16-wide tile's second four) have nothing to do.
            if (part < kSplit) {
                uint32_t ra[16], rb[16];
                tc::tmem_ld16_issue(trow + 16 * j_lo, ra);
                tc::tmem_wait16(ra);
#pragma unroll 1
                for (int j = j_lo; j < j_hi; j += 2) {
                    if (j + 1 < j_hi) tc::tmem_ld16_issue(trow + 16 * (j + 1), rb);
                    process(j, ra);
                    if (j + 1 >= j_hi) break;
                    tc::tmem_wait16(rb);
                    if (j + 2 < j_hi) tc::tmem_ld16_issue(trow + 16 * (j + 2), ra);
                    process(j + 1, rb);
                    if (j + 2 < j_hi) tc::tmem_wait16(ra);
                }
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, kCols);
}

// ---- persistent hidden-layer GEMM (width 256) ----
// Y[rows x 256] = A[rows x K] W^T with the hidden layers' epilogues (kBiasSilu, kDsilu), one CTA per SM
// for the whole batch. CTA pairs split the 256 output columns into two 128-wide halves, and each CTA
// keeps its half's weights [128 x K] resident in shared memory for all of its row tiles. Warp roles:
// warp 8 lane 0 streams the 128 x 64 chunks of A through a 4-stage TMA ring; warp 9 lane 0 issues the
// MMAs (128 x 128 x 16) into one of two TMEM accumulators, so that a tile's MMAs overlap the previous
// tile's epilogue; warps 0-7 run the staged epilogue (warp w: TMEM lane quadrant w & 3, columns
// 64 (w >> 2) .. + 63 of the half) and hand the accumulator back. Every wait is bounded; after a
// timeout the roles stop, the loads in flight are waited for (bounded) and the error flag is set.
constexpr int kLayerN = 128;                  // output columns per CTA
constexpr int kLayerEpiWarps = 8;
constexpr int kLayerThreads = 32 * (kLayerEpiWarps + 2);
constexpr int kLayerWBytes = 4 * kLayerN * kChunkK * 2;  // K <= 256: four 16 KB chunks of W
// Ring stages (16 KB each) and staging per epilogue warp: the forward kernel writes its Z and A boxes
// one after the other through one 4 KB box and keeps eight chunks (two tiles of A) in flight; the
// input-gradient kernel double-buffers its Z / dZ boxes (8 KB) and streams the fused weight gradient's
// operand through its six stages too.
__host__ __device__ constexpr int layer_ring(int epi) { return epi == 1 /* kBiasSilu */ ? 8 : 6; }
__host__ __device__ constexpr int layer_stage(int epi) { return epi == 1 /* kBiasSilu */ ? 4096 : 8192; }

__host__ __device__ constexpr int layer_smem_bytes(int epi) {
    return kLayerWBytes + layer_ring(epi) * kABytes + kLayerEpiWarps * layer_stage(epi) + 1024 /* alignment */ +
           512 /* barriers */ + kLayerN * 4 /* bias or column sums */;
}

// WG > 0 (kDsilu only): the kernel also computes the weight gradient of the layer whose dZ it produces,
// dW[n0 + i][j] += sum over the tile's rows r of dZ[r][n0 + i] Ain[r][j] (j < wg, Ain = the layer's input
// activations, row-major [rows x wg], map tmB2 in [32 rows x 64] boxes; wg = WG, or 64 when WG = 256 and
// ea.wg = 64 -- the first layer, whose input is the 64 features): per tile one more set of MMAs
// (M = 128 dZ columns, N = wg, K = the tile's 128 rows), both operands MN-major -- dZ straight from the
// epilogue's staging boxes, which are laid out as the 128-byte-swizzled MN-major operand, Ain through
// the ring (as many 32-row chunks per stage as fit: one at width 256, four at width 64) -- accumulated
// in TMEM columns 256 .. 256 + wg over all of the CTA's tiles and added into the FP32 gradient (map
// tmG) with TMA reductions at the end. The ring carries the tiles' chunks in the
// order D(0), D(1), G(0), D(2), G(1), ... (D = the layer GEMM's A, G = Ain), so that the weight
// gradient of tile t, which waits for tile t's epilogue, never holds up the MMAs of tile t + 1.
template <int EPI, int WG = 0>
__global__ void __launch_bounds__(kLayerThreads, 1)
layer_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmW,
             const __grid_constant__ CUtensorMap tmZ, const __grid_constant__ CUtensorMap tmR,
             const __grid_constant__ CUtensorMap tmB2, const __grid_constant__ CUtensorMap tmG, EpiArgs ea, int K,
             int* err) {
    static_assert(EPI == kBiasSilu || EPI == kDsilu, "hidden-layer epilogues only");
    static_assert(WG == 0 || (EPI == kDsilu && (WG == 64 || WG == 256)), "a fused weight gradient of width 64 or 256");
    static_assert(kBiasSilu == 1, "layer_ring and layer_stage name the forward epilogue by its value");
    constexpr int kLayerRing = layer_ring(EPI);
    constexpr int kLayerStage = layer_stage(EPI);
    constexpr uint32_t kIdesc = tc::idesc_bf16(kTileM, kLayerN);
    constexpr uint32_t kTmemCols = WG ? 512 : 2 * kLayerN;
    // The fused weight gradient's width: WG, or (WG = 256) the launch's 64 -- the first layer's, against the
    // 64 features -- so that every backward layer runs the same code, which the previous launch has
    // brought into the SM's caches.
    const int wg = WG == 256 && ea.wg == 64 ? 64 : WG;
    const uint32_t idescG = tc::idesc_bf16(kTileM, wg ? wg : 64, true, true);
    const int gbytes = wg * 32 * 2;                            // one 32-row chunk of Ain
    const int grows = wg ? 32 * (kABytes / gbytes) : 32;       // Ain rows per ring stage (128 at width 64)
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t* sW = smem;
    uint8_t* sRing = sW + kLayerWBytes;
    uint8_t* sStage = sRing + kLayerRing * kABytes;
    uint64_t* full = reinterpret_cast<uint64_t*>(sStage + kLayerEpiWarps * kLayerStage);
    uint64_t* empty = full + kLayerRing;
    uint64_t* tfull = empty + kLayerRing;       // accumulator b holds a finished tile
    uint64_t* tempty = tfull + 2;               // accumulator b has been read by the epilogue
    uint64_t* wbar = tempty + 2;                // the weights have landed
    uint64_t* zbar = wbar + 1;                  // [warp][buffer]: kDsilu pre-activation boxes
    uint64_t* dzready = zbar + 2 * kLayerEpiWarps;  // (WG) staging buffer b holds a tile's dZ
    uint64_t* dzfree = dzready + 2;                 // (WG) the weight-gradient MMAs have read buffer b
    uint64_t* wdone = dzfree + 2;                   // (WG) every weight-gradient MMA has completed
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(wdone + 1);
    volatile int* fail = reinterpret_cast<volatile int*>(tmem_slot + 1);
    float* sx = reinterpret_cast<float*>(reinterpret_cast<uint8_t*>(full) + 512);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nh = ea.N / kLayerN;                       // column halves (2)
    const int n0 = (blockIdx.x % nh) * kLayerN;
    const int pairs = gridDim.x / nh;
    const int pair = blockIdx.x / nh;
    const int mtiles = (ea.M + kTileM - 1) / kTileM;
    const int my_tiles = pair < mtiles ? (mtiles - pair + pairs - 1) / pairs : 0;  // tiles pair, pair + pairs, ...
    const int kc = (K + kChunkK - 1) / kChunkK;          // K chunks (<= 4)

    if (threadIdx.x == 0) {
        for (int s = 0; s < kLayerRing; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&tfull[b], 1);
            tc::mbar_init(&tempty[b], kLayerEpiWarps);
        }
        tc::mbar_init(wbar, 1);
        for (int i = 0; i < 2 * kLayerEpiWarps; ++i) tc::mbar_init(&zbar[i], 1);
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&dzready[b], kLayerEpiWarps);
            tc::mbar_init(&dzfree[b], 1);
        }
        tc::mbar_init(wdone, 1);
        *fail = 0;
        tc::fence_mbar_init();
    }
    if (warp == kLayerEpiWarps + 1) tc::tmem_alloc(tmem_slot, kTmemCols);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    // The weights are loaded before the wait on the previous grid, overlapping its tail, unless the
    // previous kernel wrote them (late_weights): otherwise they were written by the optimiser step (or a
    // weight upload) at least two launches upstream, and no kernel in between writes them.
    auto load_weights = [&]() {
        if (warp == kLayerEpiWarps && lane == 0) {
            tc::mbar_expect_tx(wbar, kc * kABytes);
            for (int c = 0; c < kc; ++c) tc::tma_load_2d(sW + c * kABytes, &tmW, c * kChunkK, n0, wbar);
        }
        if constexpr (EPI == kBiasSilu) {  // the biases too, or the zeroed bias-gradient sums
            for (int i = threadIdx.x; i < kLayerN; i += blockDim.x) sx[i] = ea.bias[n0 + i];
        } else {
            for (int i = threadIdx.x; i < kLayerN; i += blockDim.x) sx[i] = 0.0f;
        }
    };
    if (!ea.late_weights) load_weights();
    int pre_issued = 0;  // (producer) A chunks issued before the launch wait, into the fresh ring stages
    if constexpr (EPI == kBiasSilu) {
        if (ea.early_a && warp == kLayerEpiWarps && lane == 0) {
            for (; pre_issued < kLayerRing && pre_issued < my_tiles * kc; ++pre_issued) {
                const int t = pre_issued / kc, c = pre_issued % kc;
                tc::mbar_expect_tx(&full[pre_issued], kABytes);
                tc::tma_load_2d(sRing + pre_issued * kABytes, &tmA, c * kChunkK, (pair + t * pairs) * kTileM,
                                &full[pre_issued]);
            }
        }
    }
    // So is each epilogue warp's first pre-activation box (kDsilu): Z was written by the forward pass.
    if constexpr (EPI == kDsilu) {
        if (warp < kLayerEpiWarps && lane == 0 && my_tiles > 0) {
            tc::mbar_expect_tx(&zbar[2 * warp], 4096);
            tc::tma_load_2d(sStage + warp * kLayerStage, &tmZ, n0 + 64 * (warp >> 2), pair * kTileM + 32 * (warp & 3),
                            &zbar[2 * warp]);
        }
    }
    // Launched programmatically: the previous grid of the stream has finished before any other global
    // access.
    tc::grid_dep_wait();
    tc::grid_dep_launch();
    if (ea.late_weights) load_weights();
    __syncthreads();

    if (warp == kLayerEpiWarps) {
        // ---- producer: the A chunks of every tile through the ring (the weights are on their way) ----
        if (lane == 0) {
            int issued = pre_issued;
            // Takes the next ring stage (false: a wait timed out).
            auto next_stage = [&](int& s) {
                s = issued % kLayerRing;
                if (!tc::mbar_wait(&empty[s], ((issued / kLayerRing) & 1) ^ 1)) {
                    *fail = 1;
                    return false;
                }
                return true;
            };
            bool ok = true;
            for (int t = 0; t <= my_tiles && ok && !*fail; ++t) {
                if (t < my_tiles) {  // D(t): the layer GEMM's A chunks
                    const int m0 = (pair + t * pairs) * kTileM;
                    for (int c = 0; c < kc && ok; ++c) {
                        if (t * kc + c < pre_issued) continue;  // loaded before the launch wait
                        int s;
                        if (!(ok = next_stage(s))) break;
                        tc::mbar_expect_tx(&full[s], kABytes);
                        tc::tma_load_2d(sRing + s * kABytes, &tmA, c * kChunkK, m0, &full[s]);
                        ++issued;
                    }
                }
                if constexpr (WG > 0) {
                    if (t >= 1 && ok) {  // G(t - 1): the weight gradient's Ain rows, grows per stage
                        const int m0 = (pair + (t - 1) * pairs) * kTileM;
                        for (int c = 0; c < kTileM / grows && ok; ++c) {
                            int s;
                            if (!(ok = next_stage(s))) break;
                            tc::mbar_expect_tx(&full[s], (grows / 32) * gbytes);
                            for (int q = 0; q < grows / 32; ++q)
                                for (int j = 0; j < wg / 64; ++j)
                                    tc::tma_load_2d(sRing + s * kABytes + q * gbytes + j * 4096, &tmB2, 64 * j,
                                                    m0 + grows * c + 32 * q, &full[s]);
                            ++issued;
                        }
                    }
                }
            }
            // Drain (bounded): every chunk issued has landed before the CTA may exit. A stage is refilled
            // only after its previous chunk was consumed, so only the last kLayerRing chunks can still be
            // in flight, each the latest phase of its stage.
            if (!tc::mbar_wait(wbar, 0)) *fail = 1;
            for (int q = issued > kLayerRing ? issued - kLayerRing : 0; q < issued; ++q)
                tc::mbar_wait(&full[q % kLayerRing], (q / kLayerRing) & 1);
        }
    } else if (warp == kLayerEpiWarps + 1) {
        // ---- MMA issuer ----
        if (lane == 0) {
            bool ok = tc::mbar_wait(wbar, 0);
            int taken = 0;
            // The next ring stage, once its chunk has landed (false: the wait timed out). The chunk came
            // by TMA, whose completion on the barrier orders it before the MMAs; the other roles' failures
            // are checked once per tile.
            auto take = [&](int& s) {
                s = taken % kLayerRing;
                return tc::mbar_wait(&full[s], (taken / kLayerRing) & 1);
            };
            for (int t = 0; t <= my_tiles && ok; ++t) {
                if (t < my_tiles) {  // D(t) into accumulator t & 1
                    const int b = t & 1, u = t >> 1;
                    ok = tc::mbar_wait(&tempty[b], (u & 1) ^ 1) && !*fail;
                    tc::fence_after_sync();
                    const uint32_t d = tmem + b * kLayerN;
                    for (int c = 0; c < kc && ok; ++c) {
                        int s;
                        if (!(ok = take(s))) break;
                        const uint64_t ad = tc::smem_desc_sw128(sRing + s * kABytes);
                        const uint64_t bd = tc::smem_desc_sw128(sW + c * kABytes);
#pragma unroll
                        for (int kk = 0; kk < kChunkK / 16; ++kk)
                            tc::mma_bf16(d, ad + 2 * kk, bd + 2 * kk, kIdesc, (c > 0 || kk > 0) ? 1u : 0u);
                        tc::mma_commit(&empty[s]);
                        ++taken;
                    }
                    if (ok) tc::mma_commit(&tfull[b]);
                }
                if constexpr (WG > 0) {
                    if (t >= 1 && ok) {  // G(t - 1): dW += dZ(t - 1)^T Ain(t - 1), K = 16 rows per MMA
                        const int tg = t - 1, b = tg & 1;
                        ok = tc::mbar_wait(&dzready[b], (tg >> 1) & 1) && !*fail;
                        tc::fence_after_sync();
                        for (int c = 0; c < kTileM / grows && ok; ++c) {
                            int s;
                            if (!(ok = take(s))) break;
                            for (int q = 0; q < grows / 32; ++q) {
                                const int r32 = c * (grows / 32) + q;  // rows 32 r32 .. + 31: quad r32's boxes
#pragma unroll
                                for (int h = 0; h < 2; ++h) {
                                    // dZ: M = the CTA's 128 columns (part 0 and part 1 boxes, 4 warps apart)
                                    const uint64_t ad = tc::smem_desc_sw128_mn(
                                        sStage + r32 * kLayerStage + b * 4096 + h * 2048, 4 * kLayerStage);
                                    const uint64_t bd =
                                        tc::smem_desc_sw128_mn(sRing + s * kABytes + q * gbytes + h * 2048, 4096);
                                    tc::mma_bf16(tmem + 2 * kLayerN, ad, bd, idescG,
                                                 (tg > 0 || r32 > 0 || h > 0) ? 1u : 0u);
                                }
                            }
                            tc::mma_commit(&empty[s]);
                            ++taken;
                        }
                        if (ok) tc::mma_commit(&dzfree[b]);
                    }
                }
            }
            if constexpr (WG > 0) {
                if (ok) tc::mma_commit(wdone);
            }
            if (!ok) {
                *fail = 1;
                // the MMAs already issued complete in order: wait (bounded) for the last one's commit
                if (taken > 0) tc::mbar_wait(&empty[(taken - 1) % kLayerRing], ((taken - 1) / kLayerRing) & 1);
            }
        }
    } else {
        // ---- epilogue warps ----
        const int quad = warp & 3, part = warp >> 2;
        uint8_t* wb = sStage + warp * kLayerStage;
        const int sw = lane & 7;
        const uint32_t tq = tmem + (static_cast<uint32_t>(32 * quad) << 16) + 64 * part;
        const int x = n0 + 64 * part;  // the warp's first output column
        bool ok = true;
        // kDsilu: pre-activation box loads (lane 0 issues; tile 0's before the launch wait)
        int z_issued = EPI == kDsilu && my_tiles > 0 ? 1 : 0, z_waited = 0;
        // kDsilu: this lane's share of the bias gradient of the warp's 64 columns, summed over the rows it
        // meets in all of the CTA's tiles (the CTA's columns are the same for every tile); the sums over
        // the warp's lanes are taken once, after the last tile.
        float csum[64];
#pragma unroll
        for (int i = 0; i < 64; ++i) csum[i] = 0.0f;
        auto load_z = [&](int t) {      // the box of tile t into buffer t & 1 (lane 0)
            uint64_t* bar = &zbar[2 * warp + (t & 1)];
            tc::mbar_expect_tx(bar, 4096);
            tc::tma_load_2d(wb + (t & 1) * 4096, &tmZ, x, (pair + t * pairs) * kTileM + 32 * quad, bar);
            ++z_issued;
        };
        for (int t = 0; t < my_tiles; ++t) {
            const int b = t & 1, u = t >> 1;
            const int y0 = (pair + t * pairs) * kTileM + 32 * quad;
            const bool live = y0 + lane < ea.M;
            if (lane == 0) tc::bulk_wait_read_all();  // the stores of tile t - 1 have read the staging
            if constexpr (EPI == kDsilu && WG == 0) {
                if (lane == 0 && t + 1 < my_tiles) load_z(t + 1);  // one tile ahead, into the other buffer
            }
            __syncwarp();
            ok = __all_sync(0xffffffffu, tc::mbar_wait(&tfull[b], u & 1) ? 1 : 0) != 0 && !*fail;
            if constexpr (EPI == kDsilu) {
                if (ok) {
                    ok = __all_sync(0xffffffffu, tc::mbar_wait(&zbar[2 * warp + (t & 1)], (t >> 1) & 1) ? 1 : 0) != 0;
                    if (ok) ++z_waited;
                }
            }
            if (!ok) break;
            tc::fence_after_sync();
            // The tile's 64 columns at once; the accumulator goes back to the MMA thread right away.
            uint32_t ra[32], rb[32];
            tc::tmem_ld32_issue(tq + b * kLayerN, ra);
            tc::tmem_ld32_issue(tq + b * kLayerN + 32, rb);
            tc::tmem_wait32(ra);
            tc::tmem_wait32(rb);
            tc::fence_before_sync();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&tempty[b]);
            if constexpr (WG > 0) {
                // The next tile's Z box as early as its buffer (tile t - 1's) is free: if the weight-gradient
                // MMAs have read it by now, issue the load here; else at the end of this iteration.
                if (lane == 0 && t + 1 < my_tiles && z_issued == t + 1 &&
                    (t == 0 || tc::mbar_test(&dzfree[(t - 1) & 1], ((t - 1) >> 1) & 1)))
                    load_z(t + 1);
            }
            uint8_t* zin = wb + (t & 1) * 4096;
            uint4 av[8];  // kBiasSilu: the tile's A values (BF16) wait here while the Z box is stored
#pragma unroll
            for (int g = 0; g < 4; ++g) {
                const uint32_t* r = g < 2 ? ra + 16 * g : rb + 16 * (g - 2);
                const int cb = 64 * part + 16 * g;  // column within the CTA's half
                __align__(16) bf16 ob[16];
                if constexpr (EPI == kBiasSilu) {
                    __align__(16) bf16 zb[16];
#pragma unroll
                    for (int i = 0; i < 16; i += 2) {
                        const float z0 = __uint_as_float(r[i]) + sx[cb + i];
                        const float z1 = __uint_as_float(r[i + 1]) + sx[cb + i + 1];
                        zb[i] = __float2bfloat16_rn(z0);
                        zb[i + 1] = __float2bfloat16_rn(z1);
                        *reinterpret_cast<uint32_t*>(&ob[i]) = silu2_half(0.5f * z0, 0.5f * z1);
                    }
                    uint4* zrow = reinterpret_cast<uint4*>(wb + lane * 128);
                    zrow[(2 * g) ^ sw] = reinterpret_cast<const uint4*>(zb)[0];
                    zrow[(2 * g + 1) ^ sw] = reinterpret_cast<const uint4*>(zb)[1];
                    av[2 * g] = reinterpret_cast<const uint4*>(ob)[0];
                    av[2 * g + 1] = reinterpret_cast<const uint4*>(ob)[1];
                } else {
                    uint4* zrow = reinterpret_cast<uint4*>(zin + lane * 128);
                    __align__(16) bf16 zv[16];
                    reinterpret_cast<uint4*>(zv)[0] = zrow[(2 * g) ^ sw];
                    reinterpret_cast<uint4*>(zv)[1] = zrow[(2 * g + 1) ^ sw];
                    float dz[16];
#pragma unroll
                    for (int i = 0; i < 16; ++i) {
                        const float z = __bfloat162float(zv[i]);
                        const float sg = sigmoidf(z);
                        dz[i] = live ? __uint_as_float(r[i]) * sg * (1.0f + z * (1.0f - sg)) : 0.0f;
                        ob[i] = __float2bfloat16_rn(dz[i]);
                    }
                    zrow[(2 * g) ^ sw] = reinterpret_cast<const uint4*>(ob)[0];
                    zrow[(2 * g + 1) ^ sw] = reinterpret_cast<const uint4*>(ob)[1];
#pragma unroll
                    for (int i = 0; i < 16; ++i) csum[16 * g + i] += dz[i];
                }
            }
            tc::fence_proxy_async();
            __syncwarp();
            if constexpr (EPI == kBiasSilu) {
                // Z leaves first; once the TMA unit has read the box, A goes through the same box.
                if (lane == 0) {
                    tc::tma_store_2d(&tmZ, wb, x, y0);
                    tc::bulk_commit();
                    tc::bulk_wait_read_all();
                }
                __syncwarp();
                uint4* arow = reinterpret_cast<uint4*>(wb + lane * 128);
#pragma unroll
                for (int c = 0; c < 8; ++c) arow[c ^ sw] = av[c];
                tc::fence_proxy_async();
                __syncwarp();
            }
            if (lane == 0) {
                if constexpr (EPI == kBiasSilu) {
                    tc::tma_store_2d(&tmR, wb, x, y0);
                } else {
                    if (!ea.no_store) tc::tma_store_2d(&tmR, zin, x, y0);
                }
                tc::bulk_commit();
                if constexpr (WG > 0) tc::mbar_arrive(&dzready[t & 1]);  // dZ(t) for the weight-gradient MMAs
            }
            if constexpr (WG > 0) {
                // The next tile's Z box goes into the buffer of tile t - 1 once the weight-gradient MMAs have
                // read it (its dZ store has: the wait at the top of this iteration).
                if (t + 1 < my_tiles) {
                    int zok = 1;
                    if (lane == 0 && z_issued == t + 1) {
                        if (t >= 1) zok = tc::mbar_wait(&dzfree[(t - 1) & 1], ((t - 1) >> 1) & 1) ? 1 : 0;
                        if (zok) load_z(t + 1);
                    }
                    if (!__shfl_sync(0xffffffffu, zok, 0)) {
                        ok = false;
                        break;
                    }
                }
            }
        }
        if constexpr (EPI == kDsilu) {
            if (ea.colsum) {
#pragma unroll
                for (int g = 0; g < 4; ++g) {
                    float v[16];
#pragma unroll
                    for (int i = 0; i < 16; ++i) v[i] = csum[16 * g + i];
                    int col;
                    const float tot = warp_colsum16(v, lane, col);
                    if (!(lane & 1)) atomicAdd(&sx[64 * part + 16 * g + col], tot);
                }
            }
        }
        if constexpr (WG > 0) {
            // The CTA's weight-gradient rows n0 .. n0 + 127 (the lanes of TMEM columns 256 ..): warp (quad,
            // part) adds rows n0 + 32 quad .. and columns part WG / 2 .. into the FP32 gradient, a [32 x 32]
            // box at a time through its (now idle) staging, double-buffered.
            if (ok) {
                if (lane == 0) tc::bulk_wait_all();
                __syncwarp();
                ok = __all_sync(0xffffffffu, tc::mbar_wait(wdone, 0) ? 1 : 0) != 0;
            }
            if (ok) {
                tc::fence_after_sync();
                const int colsw = wg / 2;
                const uint32_t trow = tmem + (static_cast<uint32_t>(32 * quad) << 16) + 2 * kLayerN + part * colsw;
#pragma unroll 1
                for (int j = 0; j < colsw / 32; ++j) {
                    uint32_t r[32];
                    tc::tmem_ld32_issue(trow + 32 * j, r);
                    tc::tmem_wait32(r);
                    uint8_t* box = wb + (j & 1) * 4096;
                    if (j >= 2) {
                        if (lane == 0) tc::bulk_wait_read_but_one();
                        __syncwarp();
                    }
                    uint4* row = reinterpret_cast<uint4*>(box + lane * 128);
#pragma unroll
                    for (int c = 0; c < 8; ++c) row[c ^ sw] = make_uint4(r[4 * c], r[4 * c + 1], r[4 * c + 2], r[4 * c + 3]);
                    tc::fence_proxy_async();
                    __syncwarp();
                    if (lane == 0) {
                        tc::tma_reduce_add_2d(&tmG, box, part * colsw + 32 * j, n0 + 32 * quad);
                        tc::bulk_commit();
                    }
                }
            }
        }
        if (lane == 0) {
            tc::bulk_wait_all();
            if (!ok) {
                *fail = 1;
                // pre-activation loads still in flight land before the CTA may exit (bounded)
                for (int j = z_waited; j < z_issued; ++j) tc::mbar_wait(&zbar[2 * warp + (j & 1)], (j >> 1) & 1);
            }
        }
    }
    __syncwarp();
    if constexpr (EPI == kDsilu) {
        __syncthreads();
        if (ea.colsum && !*fail)
            for (int i = threadIdx.x; i < kLayerN; i += blockDim.x) atomicAdd(&ea.colsum[n0 + i], sx[i]);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x == 0 && *fail) atomicExch(err, 1);
    if (warp == kLayerEpiWarps + 1) tc::tmem_dealloc(tmem, kTmemCols);
}

// The training head of the width-256 network, forward and weight gradient in one pass over A3 (the last
// hidden layer's activations, [rows x 256] row-major): per 128-row tile, Y = A3 W5^T + b5 (MMAs against
// the resident W5, TMEM columns 16 b), the rows' loss terms and dLoss/dY (to dy_rm, which the input
// gradient reads), and dW5^T += A3^T dY from the same tile in shared memory -- A3 as an MN-major operand
// straight from its K-major chunks, dY^T staged by the epilogue as a K-major [16 x 128] operand --
// accumulated in TMEM columns 32-63 over the CTA's tiles and added into the FP32 gradient with TMA
// reductions at the end. The MMA thread runs Y(t) before the weight gradient of tile t - 1, so that tile
// t's epilogue overlaps it. Persistent: CTA c takes tiles c, c + grid, ..., three A3 tiles in flight;
// warp 0 loads, warp 1 issues, warps 2-9 are the epilogue in two groups of four (one warp per TMEM lane
// quadrant) that take the even and the odd tiles, so that two tiles' epilogues overlap.
constexpr int kHeadThreads = 32 * 10;
constexpr int kHeadTileBytes = 4 * kABytes;  // 128 rows x 256 BF16, four [128 x 64] chunks
constexpr int kHeadBufs = 3;                 // A3 tiles in flight per CTA
constexpr int kHeadW5Bytes = 16 * 64 * 2;    // one [16 x 64] chunk of W5 (or of dY^T)
constexpr int kHeadSmem = kHeadBufs * kHeadTileBytes + 4 * kHeadW5Bytes + 2 * 2 * kHeadW5Bytes + 1024 /* alignment */ + 256 +
                          8 * 20 * 4 + 256;

__global__ void __launch_bounds__(kHeadThreads, 1)
head_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmW,
            const __grid_constant__ CUtensorMap tmG, EpiArgs ea, int* err) {
    constexpr uint32_t kIdY = tc::idesc_bf16(kTileM, 16);              // Y: A3 (K-major) x W5^T
    constexpr uint32_t kIdG = tc::idesc_bf16(kTileM, 16, true, false);  // dW5^T: A3^T (MN-major) x dY
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t* sA = smem;                          // kHeadBufs A3 tiles
    uint8_t* sW = sA + kHeadBufs * kHeadTileBytes;  // W5, four K chunks
    uint8_t* sD = sW + 4 * kHeadW5Bytes;         // dY^T, two buffers of two K chunks
    uint64_t* full = reinterpret_cast<uint64_t*>(sD + 4 * kHeadW5Bytes);
    uint64_t* empty = full + kHeadBufs;  // the tile's MMAs (Y and weight gradient) have read A3 buffer a
    uint64_t* yfull = empty + kHeadBufs;  // Y of tile t is in TMEM columns 16 (t & 1)
    uint64_t* yempty = yfull + 2;  // the epilogue has read it
    uint64_t* dyready = yempty + 2;
    uint64_t* dyfree = dyready + 2;
    uint64_t* wbar = dyfree + 2;
    uint64_t* wdone = wbar + 1;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(wdone + 1);
    volatile int* fail = reinterpret_cast<volatile int*>(tmem_slot + 1);
    float* red = reinterpret_cast<float*>(reinterpret_cast<uint8_t*>(full) + 256);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ntiles = (ea.M + kTileM - 1) / kTileM;
    const int my = static_cast<int>(blockIdx.x) < ntiles ? (ntiles - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;
    if (threadIdx.x == 0) {
        for (int a = 0; a < kHeadBufs; ++a) {
            tc::mbar_init(&full[a], 1);
            tc::mbar_init(&empty[a], 1);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&yfull[b], 1);
            tc::mbar_init(&yempty[b], 4);
            tc::mbar_init(&dyready[b], 4);
            tc::mbar_init(&dyfree[b], 1);
        }
        tc::mbar_init(wbar, 1);
        tc::mbar_init(wdone, 1);
        *fail = 0;
        tc::fence_mbar_init();
    }
    if (warp == 1) tc::tmem_alloc(tmem_slot, 64);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    // W5 before the wait on the previous grid (written by the optimiser step, launches upstream).
    if (warp == 0 && lane == 0 && my > 0) {
        tc::mbar_expect_tx(wbar, 4 * kHeadW5Bytes);
        for (int c = 0; c < 4; ++c) tc::tma_load_2d(sW + c * kHeadW5Bytes, &tmW, 64 * c, 0, wbar);
    }
    tc::grid_dep_wait();
    tc::grid_dep_launch();

    if (warp == 0) {
        if (lane == 0 && my > 0) {  // ---- producer: the A3 tiles through kHeadBufs buffers
            int t = 0;
            for (; t < my && !*fail; ++t) {
                const int a = t % kHeadBufs;
                if (!tc::mbar_wait(&empty[a], ((t / kHeadBufs) & 1) ^ 1)) {
                    *fail = 1;
                    break;
                }
                const int m0 = (blockIdx.x + t * gridDim.x) * kTileM;
                tc::mbar_expect_tx(&full[a], kHeadTileBytes);
                for (int c = 0; c < 4; ++c) tc::tma_load_2d(sA + a * kHeadTileBytes + c * kABytes, &tmA, 64 * c, m0, &full[a]);
            }
            // Drain (bounded): the loads issued have landed before the CTA may exit (the last kHeadBufs,
            // each the latest phase of its buffer).
            tc::mbar_wait(wbar, 0);
            for (int q = t > kHeadBufs ? t - kHeadBufs : 0; q < t; ++q)
                tc::mbar_wait(&full[q % kHeadBufs], (q / kHeadBufs) & 1);
        }
    } else if (warp == 1) {
        if (lane == 0 && my > 0) {  // ---- MMA issuer: Y(t), then the weight gradient of tile t - 1
            bool ok = tc::mbar_wait(wbar, 0);
            for (int t = 0; t <= my && ok; ++t) {
                if (t < my) {
                    const int a = t % kHeadBufs, b = t & 1;
                    ok = tc::mbar_wait(&full[a], (t / kHeadBufs) & 1) && tc::mbar_wait(&yempty[b], ((t >> 1) & 1) ^ 1) &&
                         !*fail;
                    if (!ok) break;
                    tc::fence_after_sync();
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        const uint64_t ad = tc::smem_desc_sw128(sA + a * kHeadTileBytes + c * kABytes);
                        const uint64_t bd = tc::smem_desc_sw128(sW + c * kHeadW5Bytes);
#pragma unroll
                        for (int kk = 0; kk < 4; ++kk)
                            tc::mma_bf16(tmem + 16 * b, ad + 2 * kk, bd + 2 * kk, kIdY, (c | kk) ? 1u : 0u);
                    }
                    tc::mma_commit(&yfull[b]);
                }
                if (t >= 1) {
                    const int tg = t - 1, a = tg % kHeadBufs, b = tg & 1;
                    ok = tc::mbar_wait(&dyready[b], (tg >> 1) & 1) && !*fail;
                    if (!ok) break;
                    tc::fence_after_sync();
#pragma unroll
                    for (int p = 0; p < 2; ++p)      // A3 columns 128 p .. 128 p + 127 (chunks 2 p, 2 p + 1)
#pragma unroll
                        for (int kk = 0; kk < 8; ++kk) {  // rows 16 kk .. 16 kk + 15
                            const uint64_t ad = tc::smem_desc_sw128_mn(
                                sA + a * kHeadTileBytes + 2 * p * kABytes + kk * 2048, kABytes);
                            const uint64_t bd = tc::smem_desc_sw128(sD + b * 2 * kHeadW5Bytes + (kk >> 2) * kHeadW5Bytes) +
                                                2 * (kk & 3);
                            tc::mma_bf16(tmem + 32 + 16 * p, ad, bd, kIdG, (tg > 0 || kk > 0) ? 1u : 0u);
                        }
                    tc::mma_commit(&empty[a]);
                    tc::mma_commit(&dyfree[b]);
                }
            }
            if (!ok) *fail = 1;
            tc::mma_commit(wdone);  // every MMA issued has completed when this arrives
        }
    } else {
        // ---- epilogue: lane = row of the tile (warp w reads TMEM lanes 32 (w % 4) ..); group grp takes
        // the tiles t with t & 1 == grp, whose accumulator and dY^T buffers are its own
        const int quad = warp & 3, grp = (warp - 2) >> 2;
        const int row = 32 * quad + lane;
        float csum[kOutPad], tsum[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int i = 0; i < kOutPad; ++i) csum[i] = 0.0f;
        bool ok = true;
        float bias[kOutPad];  // the head's bias, once
#pragma unroll
        for (int i = 0; i < kOutPad; ++i) bias[i] = ea.bias[i];
        for (int t = grp; t < my && ok; t += 2) {
            const int b = t & 1;
            const int m = (blockIdx.x + t * gridDim.x) * kTileM + row;
            // The row's class and targets, loaded while the tile's MMAs run.
            int cl = 0;
            float tgv[kOut];
#pragma unroll
            for (int i = 0; i < kOut; ++i) tgv[i] = 0.0f;
            if (m < ea.M) {
                cl = static_cast<int>(ea.cls[m]) - 1;
                const float* tr = ea.tgt + static_cast<size_t>(m) * kOut;
                if ((reinterpret_cast<uintptr_t>(ea.tgt) & 15) == 0) {  // rows of 32 bytes from an aligned base
                    const float4 t0 = reinterpret_cast<const float4*>(tr)[0], t1 = reinterpret_cast<const float4*>(tr)[1];
                    tgv[0] = t0.x; tgv[1] = t0.y; tgv[2] = t0.z; tgv[3] = t0.w;
                    tgv[4] = t1.x; tgv[5] = t1.y; tgv[6] = t1.z; tgv[7] = t1.w;
                } else {
#pragma unroll
                    for (int i = 0; i < kOut; ++i) tgv[i] = tr[i];
                }
            }
            ok = __all_sync(0xffffffffu, tc::mbar_wait(&yfull[b], (t >> 1) & 1) ? 1 : 0) != 0 && !*fail;
            if (!ok) break;
            tc::fence_after_sync();
            uint32_t r[16];
            tc::tmem_ld16_issue(tmem + (static_cast<uint32_t>(32 * quad) << 16) + 16 * b, r);
            tc::tmem_wait16(r);
            tc::fence_before_sync();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&yempty[b]);
            float d[kOutPad], terms[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
            for (int i = 0; i < kOutPad; ++i) d[i] = 0.0f;
            if (m < ea.M) {
                float y[kOutPad];
#pragma unroll
                for (int i = 0; i < kOutPad; ++i) y[i] = __uint_as_float(r[i]) + bias[i];
                row_loss(y, cl, tgv, ea.inv_n, ea.lw, d, terms);
            }
            __align__(16) bf16 ob[kOutPad];
#pragma unroll
            for (int i = 0; i < kOutPad; ++i) {
                ob[i] = __float2bfloat16_rn(d[i]);
                csum[i] += d[i];
            }
#pragma unroll
            for (int i = 0; i < 4; ++i) tsum[i] += terms[i];
            if (m < ea.M) {
                uint4* dst = reinterpret_cast<uint4*>(ea.dy_rm + static_cast<size_t>(m) * kOutPad);
                dst[0] = reinterpret_cast<const uint4*>(ob)[0];
                dst[1] = reinterpret_cast<const uint4*>(ob)[1];
            }
            // dY^T of the tile (zeros past the last row) into buffer b once the weight gradient of tile
            // t - 2 has read it: element (output i, row) at row i, column row of the K-major operand.
            ok = __all_sync(0xffffffffu, tc::mbar_wait(&dyfree[b], ((t >> 1) & 1) ^ 1) ? 1 : 0) != 0;
            if (!ok) break;
            uint8_t* dt = sD + b * 2 * kHeadW5Bytes + (row >> 6) * kHeadW5Bytes;
#pragma unroll
            for (int i = 0; i < kOutPad; ++i)
                *reinterpret_cast<bf16*>(dt + i * 128 + ((((row & 63) >> 3) ^ (i & 7)) << 4) + ((row & 7) << 1)) = ob[i];
            tc::fence_proxy_async();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&dyready[b]);
        }
        if (!ok && lane == 0) *fail = 1;
        // The bias gradient and the loss terms of the CTA's rows: warp sums, then the eight warps.
#pragma unroll
        for (int i = 0; i < kOutPad + 4; ++i) {
            float v = i < kOutPad ? csum[i] : tsum[i - kOutPad] * ea.inv_n;
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if (lane == 0) red[(warp - 2) * (kOutPad + 4) + i] = v;
        }
        asm volatile("bar.sync 1, 256;" ::: "memory");
        if (warp == 2 && lane < kOutPad + 4 && !*fail && my > 0) {
            float v = 0.0f;
            for (int q = 0; q < 8; ++q) v += red[q * (kOutPad + 4) + lane];
            if (lane < kOutPad) {
                if (v != 0.0f) atomicAdd(&ea.colsum[lane], v);
            } else {
                atomicAdd(&ea.loss[lane - kOutPad], v);
            }
        }
        // dW5 += the CTA's partial: TMEM lane c of columns 32 + 16 p holds dW5[.][128 p + c] (c = 32 quad +
        // lane); group p's warps stage their [16 x 32] blocks as [32 x 32] FP32 boxes (rows 16-31 lie past
        // the 16 rows of W5 and are not written) in the idle A3 buffers and add them with TMA reductions.
        if (my > 0) {
            ok = __all_sync(0xffffffffu, tc::mbar_wait(wdone, 0) ? 1 : 0) != 0 && !*fail;
            if (ok) {
                tc::fence_after_sync();
                {
                    const int p = grp;
                    uint32_t v[16];
                    tc::tmem_ld16_issue(tmem + (static_cast<uint32_t>(32 * quad) << 16) + 32 + 16 * p, v);
                    tc::tmem_wait16(v);
                    uint8_t* box = sA + (2 * quad + p) * 4096;
#pragma unroll
                    for (int i = 0; i < 16; ++i)
                        *reinterpret_cast<uint32_t*>(box + i * 128 + (((lane >> 2) ^ (i & 7)) << 4) + ((lane & 3) << 2)) = v[i];
                    tc::fence_proxy_async();
                    __syncwarp();
                    if (lane == 0) {
                        tc::tma_reduce_add_2d(&tmG, box, 128 * p + 32 * quad, 0);
                        tc::bulk_commit();
                    }
                }
                if (lane == 0) tc::bulk_wait_all();
            } else if (lane == 0) {
                *fail = 1;
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x == 0 && *fail) atomicExch(err, 1);
    if (warp == 1) tc::tmem_dealloc(tmem, 64);
}

// ------------------------------------------------------------------------------ host side ----

// Launch with programmatic stream serialization: the grid may be scheduled while the previous grid of
// the stream is finishing; every kernel launched this way waits for it (grid_dep_wait) before it
// touches global memory, so only its set-up (barriers, TMEM) overlaps.
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at{};
    at.id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at.val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = &at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        else
            cudaGetLastError();
    });
    return fn;
}

// Tensor map of a row-major BF16 matrix [rows x cols] read in boxes of box_rows x 64 (128-byte
// swizzle; reads past the matrix are zero).
bool make_tmap_box(CUtensorMap* map, const void* base, uint64_t rows, uint64_t cols, uint32_t box_cols,
                   uint32_t box_rows, bool swizzle128) {
    auto fn = encode_fn();
    if (!fn) return false;
    if ((reinterpret_cast<uintptr_t>(base) & 15) || ((cols * 2) & 15)) return false;
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {cols * 2};
    const cuuint32_t box[2] = {box_cols, box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool make_tmap(CUtensorMap* map, const void* base, uint64_t rows, uint64_t cols, uint32_t box_rows) {
    return make_tmap_box(map, base, rows, cols, kChunkK, box_rows, true);
}

// Staged-epilogue boxes: a row-major [rows x cols] matrix in [32 rows][64 columns] boxes (128-byte
// swizzle).
bool make_tmap_rows32(CUtensorMap* map, const void* base, uint64_t rows, uint64_t cols) {
    return make_tmap_box(map, base, rows, cols, 64, 32, true);
}

// Tensor maps of the epilogue (kBiasSilu: Z and A written; kDsilu: Z read, dZ written; kReduceF32: the
// FP32 gradient, in z).
struct OutMaps {
    CUtensorMap z, r;
};

// An FP32 row-major [rows x cols] matrix in [32 rows][32 columns] boxes (128-byte swizzle), the target of
// the weight gradients' TMA reductions.
bool make_tmap_f32_32(CUtensorMap* map, const void* base, uint64_t rows, uint64_t cols) {
    auto fn = encode_fn();
    if (!fn) return false;
    if ((reinterpret_cast<uintptr_t>(base) & 15) || ((cols * 4) & 15)) return false;
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {cols * 4};
    const cuuint32_t box[2] = {32, 32};
    const cuuint32_t estr[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN, int EPI, int MAJ>
cudaError_t launch_gemm_bn(const CUtensorMap& a, const CUtensorMap& b, const EpiArgs& ea, int M, int N, int K,
                           int splits, int* err, cudaStream_t s, const OutMaps* om) {
    static std::once_flag attr;
    std::call_once(attr, [] {
        cudaFuncSetAttribute(gemm_kernel<BN, EPI, MAJ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             gemm_smem_bytes<BN, EPI>());
    });
    splits = splits < 1 ? 1 : splits;
    const int per = ((K + splits - 1) / splits + kChunkK - 1) / kChunkK * kChunkK;
    const dim3 grid((M + kTileM - 1) / kTileM, (N + BN - 1) / BN, (K + per - 1) / per);
    static const OutMaps none{};
    const OutMaps& o = om ? *om : none;
    return launch_pdl(gemm_kernel<BN, EPI, MAJ>, grid, dim3(kGemmThreads), gemm_smem_bytes<BN, EPI>(), s, a, b, o.z, o.r,
                      ea, K, per, err);
}

// C = A * B^T tile-width choice by N.
// (The hidden layers' epilogues, kBiasSilu and kDsilu, have N = the hidden width, 64 or 256, and the
// output maps; their tiles are at least 64 wide, as are those of an MN-major B.)
template <int EPI, int MAJ = 0>
cudaError_t launch_gemm(const CUtensorMap& a, const CUtensorMap& b, const EpiArgs& ea, int M, int N, int K, int splits,
                        int* err, cudaStream_t s, const OutMaps* om = nullptr) {
    if constexpr (EPI == kBiasSilu || EPI == kDsilu) {
        if (!om) return cudaErrorInvalidValue;
    }
    if constexpr (EPI == kBiasSilu || EPI == kDsilu || EPI == kReduceF32 || (MAJ & 2) != 0) {
        if (N <= 64) return launch_gemm_bn<64, EPI, MAJ>(a, b, ea, M, N, K, splits, err, s, om);
    } else {
        if (N <= 16) return launch_gemm_bn<16, EPI, MAJ>(a, b, ea, M, N, K, splits, err, s, om);
        if (N <= 64) return launch_gemm_bn<64, EPI, MAJ>(a, b, ea, M, N, K, splits, err, s, om);
    }
    return launch_gemm_bn<256, EPI, MAJ>(a, b, ea, M, N, K, splits, err, s, om);
}

int box_rows_for(int N) { return N <= 16 ? 16 : (N <= 64 ? 64 : 256); }

// The persistent hidden-layer GEMM of a width-256 network: A (rows x K, K <= 256) row-major with a
// [128 rows x 64] box map, W [256 x K] with a [128 x 64] box map, the staged epilogue's maps; one CTA per
// SM (CTA pairs over the two column halves) or fewer for small batches. WG > 0 (kDsilu): with the fused
// weight gradient of width WG (or ea.wg, 64, at WG = 256), from the input activations' [32 x 64]-box map
// `ain` into the FP32 gradient's [32 x 32]-box map `grad`.
template <int EPI, int WG = 0>
cudaError_t launch_layer(const CUtensorMap& a, const CUtensorMap& w, const OutMaps& om, const EpiArgs& ea, int K,
                         int sms, int* err, cudaStream_t s, const CUtensorMap* ain = nullptr,
                         const CUtensorMap* grad = nullptr) {
    static std::once_flag attr;
    std::call_once(attr, [] {
        cudaFuncSetAttribute(layer_kernel<EPI, WG>, cudaFuncAttributeMaxDynamicSharedMemorySize, layer_smem_bytes(EPI));
    });
    if (ea.N % kLayerN != 0 || K > 4 * kChunkK || (WG > 0 && (!ain || !grad))) return cudaErrorInvalidValue;
    static const CUtensorMap none{};
    const int nh = ea.N / kLayerN;
    const int mtiles = (ea.M + kTileM - 1) / kTileM;
    const int pairs = std::max(1, std::min(mtiles, sms / nh));
    return launch_pdl(layer_kernel<EPI, WG>, dim3(pairs * nh), dim3(kLayerThreads), layer_smem_bytes(EPI), s, a, w, om.z,
                      om.r, ain ? *ain : none, grad ? *grad : none, ea, K, err);
}

}  // namespace sur
}  // namespace bhk

using namespace bhk;
using namespace bhk::sur;

// Diagnostic: C (M x N, FP32, row-major) = A (M x K) * B (N x K)^T with A, B BF16 row-major in device
// memory, on the tensor-core GEMM kernel the surrogate uses. With splits > 1 the K range is split
// across CTAs and C is accumulated atomically (the caller zeroes it).
extern "C" bhk_status bhk_tc_gemm(const void* A, const void* B, float* C, int32_t M, int32_t N, int32_t K,
                                  int32_t splits, void* stream) {
    if (!A || !B || !C || M <= 0 || N <= 0 || K <= 0 || N > 256 || (K % 8) != 0) {
        set_last_error("bhk_tc_gemm: needs M, N, K > 0, N <= 256, K a multiple of 8");
        return BHK_EINVAL;
    }
    CUtensorMap ta, tb;
    if (!make_tmap(&ta, A, M, K, kTileM) || !make_tmap(&tb, B, N, K, box_rows_for(N))) {
        set_last_error("bhk_tc_gemm: tensor map creation failed (16-byte alignment of A, B and rows)");
        return BHK_EINVAL;
    }
    int* err = nullptr;
    if (cudaMalloc(&err, sizeof(int)) != cudaSuccess) return BHK_ENOMEM;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaMemsetAsync(err, 0, sizeof(int), s);
    EpiArgs ea{};
    ea.M = M;
    ea.N = N;
    ea.f32 = C;
    ea.ld_f32 = N;
    cudaError_t e = splits > 1 ? launch_gemm<kAtomicF32>(ta, tb, ea, M, N, K, splits, err, s)
                               : launch_gemm<kStoreF32>(ta, tb, ea, M, N, K, 1, err, s);
    int h_err = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(err);
    if (e != cudaSuccess) {
        set_last_error(std::string("bhk_tc_gemm: ") + cudaGetErrorString(e));
        return BHK_ECUDA;
    }
    if (h_err) {
        set_last_error("bhk_tc_gemm: a pipeline wait timed out");
        return BHK_ECUDA;
    }
    return BHK_OK;
}

// ============================================================================ the network ====

namespace bhk {
namespace sur {

// The hidden width (kHidden, the four SiLU layers) is a property of each network: 256 (the default) or
// 64 (a network 12.5 x cheaper to evaluate, for the speed/accuracy trade of the learned path).
constexpr int kHidDefault = 256;
__host__ __device__ constexpr bool width_ok(int hid) { return hid == 64 || hid == 256; }
__host__ __device__ constexpr int fan_in(int l, int hid) { return l == 0 ? kFeat : hid; }
__host__ __device__ constexpr int fan_out(int l, int hid) { return l == kLayers - 1 ? kOutPad : hid; }

// Flat FP32 parameter vector: W_l (fan_out x fan_in, row-major) then b_l, for l = 1..5.
struct ParamLayout {
    size_t w[kLayers], b[kLayers], total;
    explicit ParamLayout(int hid = kHidDefault) {
        size_t o = 0;
        for (int l = 0; l < kLayers; ++l) {
            w[l] = o;
            o += static_cast<size_t>(fan_out(l, hid)) * fan_in(l, hid);
            b[l] = o;
            o += fan_out(l, hid);
        }
        total = o;
    }
};

// Input normalisation to [-1, 1]: spin over [0, 0.998], inclination over [5, 89] degrees, log10 r
// over [log10 20, 3], alpha and beta over +-kImageScale M.
constexpr float kImageScale = 12.0f;

__device__ __forceinline__ void normalise(const float* x, float u[kIn]) {
    u[0] = x[0] * (2.0f / 0.998f) - 1.0f;
    u[1] = (x[1] - 0.0872664626f) * (2.0f / 1.4660765717f) - 1.0f;
    u[2] = (x[2] - 1.3010299957f) * (2.0f / 1.6989700043f) - 1.0f;
    u[3] = x[3] * (1.0f / kImageScale);
    u[4] = x[4] * (1.0f / kImageScale);
}

// Fourier features of n rays, row-major [n x 64]: lane j of a warp takes frequency j of eight
// consecutive rays (so that each ray's sines and cosines are written as two contiguous 64-byte runs),
// with the eight rays' inputs loaded up front and the lane's Fourier coefficients held in registers;
// the batch is one wave of blocks. The first kernel of a training step also zeroes what the step
// accumulates into (the gradient, n_a floats at zero_a, and the loss terms, n_b at zero_b).
constexpr int kFeatRaysPerWarp = 8;
__global__ void __launch_bounds__(256) feature_kernel(const float* __restrict__ x, const float* __restrict__ Bm,
                                                      bf16* __restrict__ rm, int n, float* zero_a, long long n_a,
                                                      float* zero_b, int n_b) {
    tc::grid_dep_wait();
    tc::grid_dep_launch();
    const long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    for (long long i = t; i < n_a; i += static_cast<long long>(gridDim.x) * blockDim.x) zero_a[i] = 0.0f;
    if (t < n_b) zero_b[t] = 0.0f;
    const long long r0 = (t >> 5) * kFeatRaysPerWarp;
    const int j = static_cast<int>(t & 31);
    if (r0 >= n) return;
    float bj[kIn];
#pragma unroll
    for (int i = 0; i < kIn; ++i) bj[i] = __ldg(&Bm[j * kIn + i]);
    float xs[kFeatRaysPerWarp][kIn];
#pragma unroll
    for (int k = 0; k < kFeatRaysPerWarp; ++k)
#pragma unroll
        for (int i = 0; i < kIn; ++i) xs[k][i] = r0 + k < n ? __ldg(x + (r0 + k) * kIn + i) : 0.0f;
#pragma unroll
    for (int k = 0; k < kFeatRaysPerWarp; ++k) {
        const long long r = r0 + k;
        if (r >= n) break;
        float u[kIn];
        normalise(xs[k], u);
        float p = 0.0f;
#pragma unroll
        for (int i = 0; i < kIn; ++i) p += bj[i] * u[i];
        // sin and cos of 2 pi p: exact reduction to r = p - rint(p) in [-1/2, 1/2], then the hardware sine
        // and cosine (absolute error ~2^-21 on [-pi, pi], far below the BF16 rounding that follows).
        float sn, cs;
        __sincosf(6.28318530717958648f * (p - rintf(p)), &sn, &cs);
        rm[r * kFeat + j] = __float2bfloat16_rn(sn);
        rm[r * kFeat + kFreq + j] = __float2bfloat16_rn(cs);
    }
}

// Blocks of feature_kernel for n rays that also zero n_a floats (at most 16 per thread).
inline unsigned feature_blocks(long long n, long long n_a) {
    const long long rays = (n + 8 * kFeatRaysPerWarp - 1) / (8 * kFeatRaysPerWarp);
    const long long zero = (n_a + 16 * 256 - 1) / (16 * 256);
    return static_cast<unsigned>(std::max<long long>(1, std::max(rays, zero)));
}

// Adam on the flat FP32 parameters; refreshes the BF16 copies W (fan_out x fan_in) and W^T.
struct AdamArgs {
    float* p;
    float* g;  // (kAdam) read, then zeroed for the next step
    float* m;
    float* v;
    bf16* w_rm[kLayers];
    bf16* w_t[kLayers];
    size_t wofs[kLayers];
    size_t total;
    int hid;                        // hidden width of the network
    float lr, b1, b2, eps, c1, c2;  // c1 = 1 / (1 - b1^t), c2 = 1 / (1 - b2^t)
    float* loss;                    // the step's four loss terms: copied to hist (if any), then zeroed
    float* hist;
};

// Weight tiles of 32 x 32 per block (the head's 16 rows in one tile row), then one block for the biases.
__host__ __device__ inline int weight_tiles(int l, int hid) {
    return ((fan_out(l, hid) + 31) / 32) * ((fan_in(l, hid) + 31) / 32);
}
__host__ __device__ inline int weights_blocks(int hid) {
    int n = 1;
    for (int l = 0; l < kLayers; ++l) n += weight_tiles(l, hid);
    return n;
}

// kAdam: one Adam step on the FP32 parameters (m, v, p), else the parameters as they are; either way
// the BF16 copies W (fan_out x fan_in) and W^T follow. A block takes a 32 x 32 tile of one layer's
// weights: 256 threads read and write the FP32 state and W along the rows (coalesced), and write W^T
// along its rows through a shared-memory transpose; the last block takes the biases. Each thread
// loads all its elements' state before it updates any (the stores may not be assumed apart from the
// next element's loads, so interleaving them would expose one load latency per element).
template <bool kAdam>
__global__ void __launch_bounds__(256) weights_kernel(AdamArgs a) {
    __shared__ bf16 tile[32][34];
    constexpr int kPer = 5;  // elements per thread (4 in a weight tile; up to 5 of the biases)
    size_t idx[kPer];
    bool in[kPer];
    float pw[kPer], gw[kPer], mw[kPer], vw[kPer];
    // Loads the state of the elements marked in[], then updates them (Adam) and stores it back. The
    // parameters and moments are loaded before the wait on the previous grid (only the optimiser step
    // writes them, a step earlier); the gradient and the loss terms after it.
    auto update_all = [&]() {
#pragma unroll
        for (int q = 0; q < kPer; ++q) {
            if (!in[q]) continue;
            pw[q] = a.p[idx[q]];
            if constexpr (kAdam) {
                mw[q] = a.m[idx[q]];
                vw[q] = a.v[idx[q]];
            }
        }
        if constexpr (kAdam) {
            tc::grid_dep_wait();
            tc::grid_dep_launch();
            if (blockIdx.x == 0 && threadIdx.x < 4 && a.loss) {
                if (a.hist) a.hist[threadIdx.x] = a.loss[threadIdx.x];
                a.loss[threadIdx.x] = 0.0f;  // for the next step, as the gradient below
            }
#pragma unroll
            for (int q = 0; q < kPer; ++q)
                if (in[q]) gw[q] = a.g[idx[q]];
#pragma unroll
            for (int q = 0; q < kPer; ++q)
                if (in[q]) a.g[idx[q]] = 0.0f;  // the next step accumulates from zero
        }
        if constexpr (kAdam) {
#pragma unroll
            for (int q = 0; q < kPer; ++q) {
                if (!in[q]) continue;
                const float g = gw[q];
                const float m = a.b1 * mw[q] + (1.0f - a.b1) * g;
                const float v = a.b2 * vw[q] + (1.0f - a.b2) * g * g;
                a.m[idx[q]] = m;
                a.v[idx[q]] = v;
                pw[q] -= a.lr * (m * a.c1) / (sqrtf(v * a.c2) + a.eps);
                a.p[idx[q]] = pw[q];
            }
        }
    };
    int b = blockIdx.x;
    int l = 0;
    for (; l < kLayers && b >= weight_tiles(l, a.hid); ++l) b -= weight_tiles(l, a.hid);
    if (l == kLayers) {  // the biases (each stored right after its layer's weights), all layers at once
        const int nb = 4 * a.hid + kOutPad;
#pragma unroll
        for (int q = 0; q < kPer; ++q) {
            const int j = threadIdx.x + q * blockDim.x;
            in[q] = j < nb;
            const int ql = j < 4 * a.hid ? j / a.hid : kLayers - 1;
            const int jj = j < 4 * a.hid ? j - ql * a.hid : j - 4 * a.hid;
            idx[q] = in[q] ? a.wofs[ql] + static_cast<size_t>(fan_out(ql, a.hid)) * fan_in(ql, a.hid) + jj : 0;
        }
        update_all();
        return;
    }
    const int fi = fan_in(l, a.hid), fo = fan_out(l, a.hid);
    const int kt = (fi + 31) / 32;
    const int o0 = (b / kt) * 32, k0 = (b % kt) * 32;
    const int c = threadIdx.x & 31, r = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < kPer; ++q) {
        const int o = o0 + r + 8 * q, k = k0 + c;
        in[q] = q < 4 && o < fo && k < fi;
        idx[q] = in[q] ? a.wofs[l] + static_cast<size_t>(o) * fi + k : 0;
    }
    update_all();
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int o = o0 + r + 8 * q, k = k0 + c;
        if (in[q]) {
            const size_t j = static_cast<size_t>(o) * fi + k;
            const bf16 wb = __float2bfloat16_rn(pw[q]);
            a.w_rm[l][j] = wb;
            tile[r + 8 * q][c] = wb;
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int k = k0 + r + 8 * q, o = o0 + c;
        if (o < fo && k < fi) a.w_t[l][static_cast<size_t>(k) * fo + o] = tile[c][r + 8 * q];
    }
}

}  // namespace sur
}  // namespace bhk

// ======================================================================= the C ABI object ====

struct bhk_surrogate {
    int device = 0;
    int cap = 0;  // batch capacity (rows of every activation buffer)
    int hid = bhk::sur::kHidDefault;  // hidden width
    int sms = 1;  // the device's SM count (grid sizes)
    bhk::sur::ParamLayout L;
    float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
    bhk::sur::bf16* w_rm[bhk::sur::kLayers] = {};
    bhk::sur::bf16* w_t[bhk::sur::kLayers] = {};
    float* Bm = nullptr;
    bhk::sur::bf16 *F_rm = nullptr, *dy_rm = nullptr, *dy_t = nullptr;
    bhk::sur::bf16 *z[4] = {}, *a_rm[4] = {}, *dz_rm[2] = {};
    float* Y = nullptr;
    float* loss = nullptr;
    int* err = nullptr;
    int64_t step = 0;
    // render scratch (grow-only)
    void* frames_dev = nullptr;
    size_t cap_frames = 0;
    int32_t* list = nullptr;
    size_t cap_list = 0;
    unsigned long long* n_list = nullptr;
    float* half_bias = nullptr;
    unsigned long long* n_list_host = nullptr;
    bhk::sur::bf16* F_all = nullptr;  // training: the features of all the batches' rows (grow-only)
    size_t cap_F_all = 0;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    float4 w = make_float4(1.0f, 10.0f, 10.0f, 10.0f);  // loss weights (CE, r_disk, ln g, direction)
    std::vector<void*> allocs;
    std::mutex mu;
};

namespace bhk {
namespace sur {

template <typename T>
bool dalloc(bhk_surrogate* s, T** p, size_t n) {
    void* q = nullptr;
    if (cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return false;
    s->allocs.push_back(q);
    *p = static_cast<T*>(q);
    return true;
}

AdamArgs adam_args(bhk_surrogate* s) {
    AdamArgs a{};
    a.p = s->p;
    a.g = s->g;
    a.m = s->m;
    a.v = s->v;
    for (int l = 0; l < kLayers; ++l) {
        a.w_rm[l] = s->w_rm[l];
        a.w_t[l] = s->w_t[l];
        a.wofs[l] = s->L.w[l];
    }
    a.total = s->L.total;
    a.hid = s->hid;
    return a;
}

struct Maps {
    CUtensorMap F_rm, dy_rm, dy_t, W[kLayers], Wt[kLayers], a_rm[4], dz_rm[2];
    CUtensorMap zs[4], as[4], dzs[2];  // the staged epilogue's [32 x 64] boxes of Z, A and dZ
    CUtensorMap Fm, am[4], dzm[2];     // F, A and dZ as MN-major operands ([64 rows x 64] boxes)
    CUtensorMap Wl[kLayers], Wtl[kLayers];  // W and W^T in [128 x 64] boxes (the persistent layer GEMM)
    CUtensorMap gm[kLayers];                // the FP32 weight gradients, targets of TMA reductions
    CUtensorMap Fs;                         // F in [32 x 64] boxes (the fused first-layer weight gradient)
};

// Tensor maps of the operands for batches of n rows (weights, features, activations, gradients), and
// with `training` also of the weight gradients' MN-major operands and of dY^T, whose rows are `cap` long
// (the K extent of the head's weight gradient, n, bounds what is read of it).
bool build_maps(bhk_surrogate* s, int n, bool training, Maps* M) {
    bool ok = make_tmap(&M->F_rm, s->F_rm, n, kFeat, kTileM) && make_tmap(&M->dy_rm, s->dy_rm, n, kOutPad, kTileM);
    for (int l = 0; l < kLayers && ok; ++l) {
        const int fi = fan_in(l, s->hid), fo = fan_out(l, s->hid);
        ok = make_tmap(&M->W[l], s->w_rm[l], fo, fi, box_rows_for(fo)) &&
             make_tmap(&M->Wt[l], s->w_t[l], fi, fo, box_rows_for(fi)) &&
             make_tmap(&M->Wl[l], s->w_rm[l], fo, fi, kLayerN) && make_tmap(&M->Wtl[l], s->w_t[l], fi, fo, kLayerN);
    }
    const int H = s->hid;
    for (int i = 0; i < 4 && ok; ++i)
        ok = make_tmap(&M->a_rm[i], s->a_rm[i], n, H, kTileM) && make_tmap_rows32(&M->zs[i], s->z[i], n, H) &&
             make_tmap_rows32(&M->as[i], s->a_rm[i], n, H);
    for (int i = 0; i < 2 && ok; ++i)
        ok = make_tmap(&M->dz_rm[i], s->dz_rm[i], n, H, kTileM) && make_tmap_rows32(&M->dzs[i], s->dz_rm[i], n, H);
    if (!training) return ok;
    ok = ok && make_tmap(&M->dy_t, s->dy_t, kOutPad, s->cap, kTileM) && make_tmap(&M->Fm, s->F_rm, n, kFeat, 64);
    for (int l = 0; l < kLayers && ok; ++l)
        ok = make_tmap_f32_32(&M->gm[l], s->g + s->L.w[l], fan_out(l, H), fan_in(l, H));
    ok = ok && make_tmap_rows32(&M->Fs, s->F_rm, n, kFeat);
    for (int i = 0; i < 4 && ok; ++i) ok = make_tmap(&M->am[i], s->a_rm[i], n, H, 64);
    for (int i = 0; i < 2 && ok; ++i) ok = make_tmap(&M->dzm[i], s->dz_rm[i], n, H, 64);
    return ok;
}

// The features' tensor maps for n rows starting at F: the first layer's [128 x 64] boxes, the fused
// first-layer weight gradient's [32 x 64] boxes and the MN-major [64 x 64] boxes.
bool feature_maps(const bf16* F, int n, Maps* M) {
    return make_tmap(&M->F_rm, F, n, kFeat, kTileM) && make_tmap_rows32(&M->Fs, F, n, kFeat) &&
           make_tmap(&M->Fm, F, n, kFeat, 64);
}

EpiArgs epi(int M, int N) {
    EpiArgs e{};
    e.M = M;
    e.N = N;
    return e;
}

// The width-256 training head (head_kernel): persistent, one CTA per SM or fewer.
cudaError_t launch_head(const Maps& M, const EpiArgs& ea, int sms, int* err, cudaStream_t s) {
    static std::once_flag attr;
    std::call_once(attr, [] {
        cudaFuncSetAttribute(head_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kHeadSmem);
    });
    const int ntiles = (ea.M + kTileM - 1) / kTileM;
    const int grid = std::max(1, std::min(ntiles, sms));
    return launch_pdl(head_kernel, dim3(grid), dim3(kHeadThreads), kHeadSmem, s, M.a_rm[3], M.W[4], M.gm[4], ea, err);
}

// Forward pass of n rows (features already in F): z, activations, and the head -- into Y, or with `loss`
// (training: the loss's targets and outputs) the loss and dLoss/dY straight from the head's epilogue;
// at width 256 the head's weight gradient too (head_kernel). late_weights: the kernel launched just
// before wrote the weights (the first layer may not load them ahead of its launch wait);
// early_features: the features were written at least two launches upstream (it may load them ahead).
cudaError_t forward(bhk_surrogate* s, const Maps& M, int n, cudaStream_t st, const EpiArgs* loss = nullptr,
                    bool late_weights = false, bool early_features = false) {
    cudaError_t e = cudaSuccess;
    const int H = s->hid;
    for (int l = 0; l < 4 && e == cudaSuccess; ++l) {
        EpiArgs ea = epi(n, H);
        ea.bias = s->p + s->L.b[l];
        ea.late_weights = l == 0 && late_weights ? 1 : 0;
        ea.early_a = l == 0 && early_features ? 1 : 0;
        OutMaps om;
        om.z = M.zs[l];
        om.r = M.as[l];
        const CUtensorMap& A = l == 0 ? M.F_rm : M.a_rm[l - 1];
        e = H == kLayerN * 2 ? launch_layer<kBiasSilu>(A, M.Wl[l], om, ea, fan_in(l, H), s->sms, s->err, st)
                             : launch_gemm<kBiasSilu>(A, M.W[l], ea, n, H, fan_in(l, H), 1, s->err, st, &om);
    }
    if (e == cudaSuccess) {
        EpiArgs ea = loss ? *loss : epi(n, kOutPad);
        ea.M = n;
        ea.N = kOutPad;
        ea.bias = s->p + s->L.b[4];
        ea.f32 = s->Y;
        ea.ld_f32 = kOutPad;
        if (!loss)
            e = launch_gemm<kStoreF32>(M.a_rm[3], M.W[4], ea, n, kOutPad, H, 1, s->err, st);
        else if (H == kLayerN * 2)
            e = launch_head(M, ea, s->sms, s->err, st);
        else
            e = launch_gemm_bn<16, kHeadLoss, 0>(M.a_rm[3], M.W[4], ea, n, kOutPad, H, 1, s->err, st, nullptr);
    }
    return e;
}

// The loss of a training batch of n rows, fused into the head's forward (targets cls and tgt).
EpiArgs loss_args(bhk_surrogate* s, const uint8_t* cls, const float* tgt, int n) {
    EpiArgs ea = epi(n, kOutPad);
    ea.cls = cls;
    ea.tgt = tgt;
    ea.dy_rm = s->dy_rm;
    ea.dy_t = s->dy_t;
    ea.ld_t = s->cap;
    ea.loss = s->loss;
    ea.inv_n = 1.0f / n;
    ea.lw = s->w;
    ea.colsum = s->g + s->L.b[4];
    return ea;
}

// K splits of a weight gradient (M x N, K = n rows): one CTA per SM over the M tiles, each split at
// least 512 rows.
int split_for(const bhk_surrogate* s, int n, int M) {
    const int mtiles = (M + kTileM - 1) / kTileM;
    long long sp = s->sms / mtiles;
    sp = std::min<long long>(sp, n / 512);
    return sp < 1 ? 1 : static_cast<int>(sp);
}

// The gradient of layer l's weights (M x N FP32 in s->g, zeroed before the backward pass) += the sum
// over K of A_k B_k^T: each K split adds its partial product with TMA reductions. MAJ as for
// gemm_kernel: the hidden layers' operands are the row-major activations and gradients themselves,
// read MN-major.
template <int MAJ>
cudaError_t weight_grad(bhk_surrogate* s, const Maps& maps, int l, const CUtensorMap& A, const CUtensorMap& B, int M,
                        int N, int K, cudaStream_t st) {
    EpiArgs ea = epi(M, N);
    OutMaps om;
    om.z = maps.gm[l];
    return launch_gemm<kReduceF32, MAJ>(A, B, ea, M, N, K, split_for(s, K, M), s->err, st, &om);
}

// Gradients of a batch of n rows (n % 128 == 0) into s->g, after forward() with the loss (which wrote
// dLoss/dY, the head's bias gradient and the loss terms). The caller has zeroed s->g and s->loss (the
// training step's feature_kernel does).
cudaError_t backward(bhk_surrogate* s, const Maps& M, int n, cudaStream_t st) {
    cudaError_t e = cudaSuccess;
    const int H = s->hid;
    // Head: dW5 = dY^T A4 (A = dY^T K-major, 16 rows; B = A4 MN-major; at width 256 head_kernel computed
    // it with the forward), then dA4 = dY W5 -> dZ4.
    if (H != kLayerN * 2) e = weight_grad<2>(s, M, 4, M.dy_t, M.am[3], kOutPad, H, n, st);
    if (e == cudaSuccess && H == kLayerN * 2) {
        // Width 256: dZ_l = (dZ_{l+1} W_{l+1}) silu'(z_l) for l = 3 .. 0 (dY W5 for l = 3), each kernel with
        // the weight gradient dW_l = dZ_l^T A_{l-1} (F for l = 0) and the bias gradient fused in; dZ_l goes
        // to buffer (3 - l) & 1, and dZ_0, which nothing reads, is not written.
        for (int l = 3; l >= 0 && e == cudaSuccess; --l) {
            EpiArgs ex = epi(n, H);
            ex.colsum = s->g + s->L.b[l];
            ex.no_store = l == 0 ? 1 : 0;
            OutMaps om;
            om.z = M.zs[l];
            om.r = M.dzs[(3 - l) & 1];
            const CUtensorMap& A = l == 3 ? M.dy_rm : M.dz_rm[(2 - l) & 1];
            const CUtensorMap& W = M.Wtl[l + 1];
            const int K = l == 3 ? kOutPad : H;
            ex.wg = l == 0 ? kFeat : kLayerN * 2;
            e = launch_layer<kDsilu, kLayerN * 2>(A, W, om, ex, K, s->sms, s->err, st, l == 0 ? &M.Fs : &M.as[l - 1],
                                                  &M.gm[l]);
        }
        return e;
    }
    if (e == cudaSuccess) {
        EpiArgs ea = epi(n, H);
        ea.colsum = s->g + s->L.b[3];
        OutMaps om;
        om.z = M.zs[3];
        om.r = M.dzs[0];
        e = launch_gemm<kDsilu>(M.dy_rm, M.Wt[4], ea, n, H, kOutPad, 1, s->err, st, &om);
    }
    // Width 64, hidden layers l = 3 .. 0: dW_l = dZ_l^T A_{l-1} (F for l = 0), dZ_{l-1} = (dZ_l W_l)
    // silu'(z_{l-1}).
    int cur = 0;
    for (int l = 3; l >= 0 && e == cudaSuccess; --l) {
        const CUtensorMap& Bop = l == 0 ? M.Fm : M.am[l - 1];
        e = weight_grad<3>(s, M, l, M.dzm[cur], Bop, H, fan_in(l, H), n, st);
        if (e != cudaSuccess || l == 0) break;
        EpiArgs ex = epi(n, H);
        ex.colsum = s->g + s->L.b[l - 1];
        OutMaps om;
        om.z = M.zs[l - 1];
        om.r = M.dzs[1 - cur];
        e = launch_gemm<kDsilu>(M.dz_rm[cur], M.Wt[l], ex, n, H, H, 1, s->err, st, &om);
        cur = 1 - cur;
    }
    return e;
}

bhk_status check_err(bhk_surrogate* s, cudaStream_t st) {
    int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, s->err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        set_last_error(std::string("surrogate: ") + cudaGetErrorString(e));
        return BHK_ECUDA;
    }
    if (h) {
        set_last_error("surrogate: a tensor-core pipeline wait timed out");
        return BHK_ECUDA;
    }
    return BHK_OK;
}

}  // namespace sur
}  // namespace bhk

extern "C" {

int64_t bhk_surrogate_num_params(void) { return static_cast<int64_t>(bhk::sur::ParamLayout().total); }

int64_t bhk_surrogate_param_count(const bhk_surrogate* s) {
    return s ? static_cast<int64_t>(s->L.total) : 0;
}

int32_t bhk_surrogate_width(const bhk_surrogate* s) { return s ? s->hid : 0; }

bhk_status bhk_surrogate_create(int device, uint64_t seed, int32_t max_batch, bhk_surrogate** out) {
    return bhk_surrogate_create_width(device, seed, max_batch, bhk::sur::kHidDefault, out);
}

bhk_status bhk_surrogate_create_width(int device, uint64_t seed, int32_t max_batch, int32_t width,
                                      bhk_surrogate** out) {
    using namespace bhk::sur;
    if (!out || max_batch <= 0 || max_batch % kTileM) {
        set_last_error("bhk_surrogate_create: max_batch must be a positive multiple of 128");
        return BHK_EINVAL;
    }
    if (!width_ok(width)) {
        set_last_error("bhk_surrogate_create_width: the hidden width must be 64 or 256");
        return BHK_EINVAL;
    }
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess) {
        set_last_error("bhk_surrogate_create: no CUDA device (no CPU fallback)");
        return BHK_ECUDA;
    }
    if (!encode_fn()) {
        set_last_error("bhk_surrogate_create: cuTensorMapEncodeTiled unavailable");
        return BHK_ECUDA;
    }
    auto* s = new bhk_surrogate();
    s->device = device;
    s->cap = max_batch;
    if (cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || s->sms < 1) s->sms = 1;
    s->hid = width;
    s->L = ParamLayout(width);
    const int H = width;
    const size_t P = s->L.total, B = static_cast<size_t>(max_batch);
    bool ok = dalloc(s, &s->p, P) && dalloc(s, &s->g, P) && dalloc(s, &s->m, P) && dalloc(s, &s->v, P) &&
              dalloc(s, &s->Bm, kFreq * kIn) && dalloc(s, &s->F_rm, B * kFeat) &&
              dalloc(s, &s->dy_rm, B * kOutPad) && dalloc(s, &s->dy_t, B * kOutPad) &&
              dalloc(s, &s->Y, B * kOutPad) && dalloc(s, &s->loss, 4) && dalloc(s, &s->err, 1) &&
              dalloc(s, &s->n_list, 1) && dalloc(s, &s->half_bias, 4 * H) &&
              cudaMallocHost(reinterpret_cast<void**>(&s->n_list_host), 8) == cudaSuccess;
    for (int i = 0; i < 3 && ok; ++i) ok = cudaEventCreate(&s->ev[i]) == cudaSuccess;
    for (int l = 0; l < kLayers && ok; ++l) {
        const size_t n = static_cast<size_t>(fan_out(l, H)) * fan_in(l, H);
        ok = dalloc(s, &s->w_rm[l], n) && dalloc(s, &s->w_t[l], n);
    }
    for (int i = 0; i < 4 && ok; ++i)
        ok = dalloc(s, &s->z[i], B * H) && dalloc(s, &s->a_rm[i], B * H);
    for (int i = 0; i < 2 && ok; ++i) ok = dalloc(s, &s->dz_rm[i], B * H);
    if (!ok) {
        bhk_surrogate_destroy(s);
        set_last_error("bhk_surrogate_create: device allocation failed");
        return BHK_ENOMEM;
    }
    // Initialisation (seeded): uniform +-sqrt(6 / fan_in) weights (He-uniform for SiLU), zero biases,
    // head scaled by 0.1.
    std::vector<float> hp(P, 0.0f);
    uint64_t st = seed ? seed : 0x9E3779B97F4A7C15ull;
    auto next = [&st]() {  // splitmix64
        uint64_t z = (st += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    auto uni = [&]() { return (next() >> 11) * (1.0 / 9007199254740992.0); };
    for (int l = 0; l < kLayers; ++l) {
        const int fi = fan_in(l, H), fo = fan_out(l, H);
        const double lim = std::sqrt(6.0 / fi) * (l == kLayers - 1 ? 0.1 : 1.0);
        for (int o = 0; o < fo; ++o)
            for (int k = 0; k < fi; ++k)
                hp[s->L.w[l] + static_cast<size_t>(o) * fi + k] =
                    (l == kLayers - 1 && o >= kOut) ? 0.0f : static_cast<float>((2.0 * uni() - 1.0) * lim);
    }
    // Fourier matrix: row j = f_j d_j with d_j a random unit direction and f_j growing geometrically
    // from 0.1 to 4 cycles per unit of the normalised input, so that smooth trends and sharp edges
    // (the shadow, the disk's rim) both have features at their scale.
    std::vector<float> hb(kFreq * kIn);
    for (int j = 0; j < kFreq; ++j) {
        double d[kIn], nrm = 0.0;
        for (int i = 0; i < kIn; ++i) {
            const double u1 = std::max(uni(), 1e-300), u2 = uni();
            d[i] = std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2);
            nrm += d[i] * d[i];
        }
        const double f = 0.1 * std::pow(40.0, static_cast<double>(j) / (kFreq - 1)) / std::sqrt(nrm);
        for (int i = 0; i < kIn; ++i) hb[j * kIn + i] = static_cast<float>(f * d[i]);
    }
    cudaError_t e = cudaMemcpy(s->p, hp.data(), P * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(s->Bm, hb.data(), hb.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(s->m, 0, P * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(s->v, 0, P * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(s->err, 0, sizeof(int));
    if (e == cudaSuccess) {
        weights_kernel<false><<<weights_blocks(s->hid), 256>>>(adam_args(s));
        e = cudaDeviceSynchronize();
    }
    if (e != cudaSuccess) {
        bhk_surrogate_destroy(s);
        set_last_error(std::string("bhk_surrogate_create: ") + cudaGetErrorString(e));
        return BHK_ECUDA;
    }
    *out = s;
    return BHK_OK;
}

bhk_status bhk_surrogate_destroy(bhk_surrogate* s) {
    if (!s) return BHK_OK;
    cudaSetDevice(s->device);
    cudaDeviceSynchronize();
    for (void* q : s->allocs) cudaFree(q);
    if (s->frames_dev) cudaFree(s->frames_dev);
    if (s->F_all) cudaFree(s->F_all);
    if (s->list) cudaFree(s->list);
    if (s->n_list_host) cudaFreeHost(s->n_list_host);
    for (cudaEvent_t e : s->ev)
        if (e) cudaEventDestroy(e);
    delete s;
    return BHK_OK;
}

bhk_status bhk_surrogate_params(bhk_surrogate* s, float* host, int32_t set) {
    if (!s || !host) return BHK_EINVAL;
    std::lock_guard<std::mutex> lock(s->mu);
    cudaSetDevice(s->device);
    const size_t bytes = s->L.total * sizeof(float);
    cudaError_t e = set ? cudaMemcpy(s->p, host, bytes, cudaMemcpyHostToDevice)
                        : cudaMemcpy(host, s->p, bytes, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && set) {
        bhk::sur::weights_kernel<false><<<bhk::sur::weights_blocks(s->hid), 256>>>(bhk::sur::adam_args(s));
        e = cudaDeviceSynchronize();
    }
    if (e != cudaSuccess) {
        set_last_error(std::string("bhk_surrogate_params: ") + cudaGetErrorString(e));
        return BHK_ECUDA;
    }
    return BHK_OK;
}

bhk_status bhk_surrogate_fourier(bhk_surrogate* s, float* host, int32_t set) {
    if (!s || !host) return BHK_EINVAL;
    std::lock_guard<std::mutex> lock(s->mu);
    cudaSetDevice(s->device);
    const size_t bytes = sizeof(float) * bhk::sur::kFreq * bhk::sur::kIn;
    const cudaError_t e = set ? cudaMemcpy(s->Bm, host, bytes, cudaMemcpyHostToDevice)
                              : cudaMemcpy(host, s->Bm, bytes, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        set_last_error(std::string("bhk_surrogate_fourier: ") + cudaGetErrorString(e));
        return BHK_ECUDA;
    }
    return BHK_OK;
}

bhk_status bhk_surrogate_loss_weights(bhk_surrogate* s, const float* w4) {
    if (!s || !w4 || !(w4[0] >= 0.0f && w4[1] >= 0.0f && w4[2] >= 0.0f && w4[3] >= 0.0f)) {
        set_last_error("bhk_surrogate_loss_weights: four non-negative weights expected");
        return BHK_EINVAL;
    }
    std::lock_guard<std::mutex> lock(s->mu);
    s->w = make_float4(w4[0], w4[1], w4[2], w4[3]);
    return BHK_OK;
}

bhk_status bhk_surrogate_adam_state(bhk_surrogate* s, float* m, float* v, int64_t* step, int32_t set) {
    if (!s || !m || !v || !step) return BHK_EINVAL;
    std::lock_guard<std::mutex> lock(s->mu);
    cudaSetDevice(s->device);
    const size_t bytes = s->L.total * sizeof(float);
    cudaError_t e;
    if (set) {
        e = cudaMemcpy(s->m, m, bytes, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(s->v, v, bytes, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) s->step = *step;
    } else {
        e = cudaMemcpy(m, s->m, bytes, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(v, s->v, bytes, cudaMemcpyDeviceToHost);
        *step = s->step;
    }
    if (e != cudaSuccess) {
        set_last_error(std::string("bhk_surrogate_adam_state: ") + cudaGetErrorString(e));
        return BHK_ECUDA;
    }
    return BHK_OK;
}

bhk_status bhk_surrogate_gradients(bhk_surrogate* s, const float* x, const uint8_t* cls, const float* tgt, int32_t n,
                                   float* grads, float* loss) {
    using namespace bhk::sur;
    if (!s || !x || !cls || !tgt || n <= 0 || n > s->cap || n % kTileM) {
        set_last_error("bhk_surrogate_gradients: n must be a multiple of 128 within the batch capacity");
        return BHK_EINVAL;
    }
    std::lock_guard<std::mutex> lock(s->mu);
    cudaSetDevice(s->device);
    Maps M;
    if (!build_maps(s, n, true, &M)) {
        set_last_error("bhk_surrogate_gradients: tensor map creation failed");
        return BHK_ECUDA;
    }
    cudaStream_t st = nullptr;
    cudaMemsetAsync(s->err, 0, sizeof(int), st);
    cudaError_t e = launch_pdl(feature_kernel, dim3(feature_blocks(n, s->L.total)), dim3(256), 0, st, x,
                               static_cast<const float*>(s->Bm), s->F_rm, n, s->g,
                               static_cast<long long>(s->L.total), s->loss, 4);
    const EpiArgs la = loss_args(s, cls, tgt, n);
    if (e == cudaSuccess) e = forward(s, M, n, st, &la);
    if (e == cudaSuccess) e = backward(s, M, n, st);
    if (e != cudaSuccess) {
        set_last_error(std::string("bhk_surrogate_gradients: ") + cudaGetErrorString(e));
        return BHK_ECUDA;
    }
    bhk_status rs = check_err(s, st);
    if (rs != BHK_OK) return rs;
    if (grads && cudaMemcpy(grads, s->g, sizeof(float) * s->L.total, cudaMemcpyDeviceToHost) != cudaSuccess)
        return BHK_ECUDA;
    if (loss && cudaMemcpy(loss, s->loss, 4 * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) return BHK_ECUDA;
    return BHK_OK;
}

bhk_status bhk_surrogate_train(bhk_surrogate* s, const float* x, const uint8_t* cls, const float* tgt, int64_t n,
                               int32_t batch, int64_t steps, float lr0, float* loss_history, void* stream) {
    using namespace bhk::sur;
    if (!s || !x || !cls || !tgt || batch <= 0 || batch > s->cap || batch % kTileM || n < batch || steps <= 0 ||
        !(lr0 > 0.0f)) {
        set_last_error("bhk_surrogate_train: bad arguments (batch a multiple of 128 within capacity, n >= batch)");
        return BHK_EINVAL;
    }
    std::lock_guard<std::mutex> lock(s->mu);
    cudaSetDevice(s->device);
    Maps M;
    if (!build_maps(s, batch, true, &M)) {
        set_last_error("bhk_surrogate_train: tensor map creation failed");
        return BHK_ECUDA;
    }
    const int64_t nb = n / batch;
    // The features of the rows of every batch the call visits (steps cycle through the nb batches), once
    // per call: the Fourier matrix does not change during training; each step reads its batch's rows at
    // their offset.
    const int64_t rows = std::min<int64_t>(nb, steps) * batch;
    if (rows > INT32_MAX) {
        set_last_error("bhk_surrogate_train: at most 2^31 - 1 training rows per call");
        return BHK_EINVAL;
    }
    if (static_cast<size_t>(rows) > s->cap_F_all) {
        if (s->F_all) cudaFree(s->F_all);
        s->F_all = nullptr;
        s->cap_F_all = 0;
        if (cudaMalloc(&s->F_all, static_cast<size_t>(rows) * kFeat * sizeof(bf16)) != cudaSuccess) {
            set_last_error("bhk_surrogate_train: out of device memory for the training features");
            return BHK_ENOMEM;
        }
        s->cap_F_all = static_cast<size_t>(rows);
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    float* hist = nullptr;
    if (loss_history && cudaMalloc(&hist, sizeof(float) * 4 * steps) != cudaSuccess) return BHK_ENOMEM;
    cudaMemsetAsync(s->err, 0, sizeof(int), st);
    cudaError_t e = cudaSuccess;
    AdamArgs aa = adam_args(s);
    aa.b1 = 0.9f;
    aa.b2 = 0.999f;
    aa.eps = 1e-8f;
    // The features' launch also zeroes the gradient and the loss terms; from then on each step's Adam
    // zeroes them after use (and copies the loss terms to the history). One step: forward, loss and
    // backward, Adam -- kernels launched programmatically back to back.
    aa.loss = s->loss;
    e = launch_pdl(feature_kernel, dim3(feature_blocks(rows, s->L.total)), dim3(256), 0, st, x,
                   static_cast<const float*>(s->Bm), s->F_all, static_cast<int>(rows), s->g,
                   static_cast<long long>(s->L.total), s->loss, 4);
    for (int64_t t = 0; t < steps && e == cudaSuccess; ++t) {
        const int64_t off = (t % nb) * batch;
        if (!feature_maps(s->F_all + off * kFeat, batch, &M)) {
            e = cudaErrorInvalidValue;
            break;
        }
        const EpiArgs la = loss_args(s, cls + off, tgt + off * kOut, batch);
        // The first layer follows the previous step's Adam, which wrote its weights; its features were
        // written by the launch before step 0 (so from step 1 on, they are launches upstream).
        if (e == cudaSuccess) e = forward(s, M, batch, st, &la, true, t > 0);
        if (e == cudaSuccess) e = backward(s, M, batch, st);
        ++s->step;
        aa.lr = static_cast<float>(0.5 * lr0 * (1.0 + std::cos(M_PI * static_cast<double>(t) / steps)));
        aa.c1 = static_cast<float>(1.0 / (1.0 - std::pow(0.9, static_cast<double>(s->step))));
        aa.c2 = static_cast<float>(1.0 / (1.0 - std::pow(0.999, static_cast<double>(s->step))));
        aa.hist = hist ? hist + 4 * t : nullptr;
        if (e == cudaSuccess) e = launch_pdl(weights_kernel<true>, dim3(weights_blocks(s->hid)), dim3(256), 0, st, aa);
    }
    bhk_status rs = e == cudaSuccess ? check_err(s, st) : BHK_ECUDA;
    if (e != cudaSuccess) set_last_error(std::string("bhk_surrogate_train: ") + cudaGetErrorString(e));
    if (hist) {
        if (rs == BHK_OK && cudaMemcpy(loss_history, hist, sizeof(float) * 4 * steps, cudaMemcpyDeviceToHost) != cudaSuccess)
            rs = BHK_ECUDA;
        cudaFree(hist);
    }
    return rs;
}

// Surrogate outputs for n rays (n x 8 FP32 per ray: 3 outcome logits, r_disk / 30, log g, escape
// unit vector) through the layer-by-layer tcgen05 GEMMs.
bhk_status bhk_surrogate_predict(bhk_surrogate* s, const float* x, int64_t n, float* out, void* stream) {
    using namespace bhk::sur;
    if (!s || !x || !out || n < 0) return BHK_EINVAL;
    std::lock_guard<std::mutex> lock(s->mu);
    cudaSetDevice(s->device);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaMemsetAsync(s->err, 0, sizeof(int), st);
    for (int64_t off = 0; off < n; off += s->cap) {
        const int rows = static_cast<int>(std::min<int64_t>(s->cap, n - off));
        Maps M;
        if (!build_maps(s, rows, false, &M)) {
            set_last_error("bhk_surrogate_predict: tensor map creation failed");
            return BHK_ECUDA;
        }
        cudaError_t e = launch_pdl(feature_kernel, dim3(feature_blocks(rows, 0)), dim3(256), 0, st, x + off * kIn,
                                   static_cast<const float*>(s->Bm), s->F_rm, rows, static_cast<float*>(nullptr),
                                   0LL, static_cast<float*>(nullptr), 0);
        if (e == cudaSuccess) e = forward(s, M, rows, st);
        if (e == cudaSuccess)
            e = cudaMemcpy2DAsync(out + off * kOut, kOut * sizeof(float), s->Y, kOutPad * sizeof(float),
                                  kOut * sizeof(float), rows, cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) {
            set_last_error(std::string("bhk_surrogate_predict: ") + cudaGetErrorString(e));
            return BHK_ECUDA;
        }
    }
    return check_err(s, st);
}

}  // extern "C"

// ====================================================== fused inference with integrator fallback ====
//
// One persistent kernel runs the whole network for 128-ray tiles: the rays' inputs come from the
// frame table (no input array), features and activations live in shared memory as the next layer's
// tcgen05 A operand (K-major, 128-byte swizzled, as TMA would have written them), accumulators in
// TMEM (256 columns per CTA, two CTAs per SM so that one CTA's epilogue overlaps the other's MMAs),
// and the weights stream from L2 through a 2-stage TMA ring in 128-row x 64-K chunks (30 per tile).
// Warp 0 loads, warp 1 issues the MMAs, warps 2-5 (one TMEM lane quadrant each, thread = ray) compute
// the features, the SiLU epilogues, the head's decode and the fallback decision, appending fallback
// rays to a list with one atomic per warp.

namespace bhk {
namespace sur {

constexpr int kCurveBins = 512;
constexpr int kCurveSamples = 2048;

// Per frame: pixel mapping, the network's per-frame inputs, and the critical curve in polar form
// about its centre (alpha_c, 0) for the band test.
struct SurFrame {
    double alpha_lo, beta_hi, px, py;
    long long offset;
    int width, height;
    float a, th, log_r, alpha_c;
    float snap;              // |alpha| below this: the axis-snap strip of kerr.h's kAxisSnap
    int curve_ok;
    float pad[2];
    // Fourier projections p_j = sum_i B_ji u_i of the frame's rays: (c_j, B_j3, B_j4) with c_j the
    // frame-constant part over u_0..u_2 (spin, inclination, log r), so that a ray's p_j is
    // fma(B_j4, u_4, fma(B_j3, u_3, c_j)) -- the same operations, in the same order, as the full sum.
    float4 proj[kFreq];
    float rho[kCurveBins];   // curve radius at psi_j = pi (j + 0.5) / kCurveBins, psi = atan2(|beta|, alpha - alpha_c)
    float kn[kCurveBins];    // rho / sqrt(rho^2 + (d rho / d psi)^2): radial offset -> normal distance
};

// Polar table of each frame's critical curve (one block per frame).
__global__ void curve_table_kernel(SurFrame* frames, const bhk_frame_desc* desc, const float* __restrict__ Bm) {
    __shared__ float sa[kCurveSamples], sbt[kCurveSamples];
    __shared__ float s_min, s_max;
    __shared__ int s_any;
    SurFrame& f = frames[blockIdx.x];
    const bhk_frame_desc d = desc[blockIdx.x];
    if (threadIdx.x < kFreq) {  // the frame's part of the Fourier projections
        const int j = threadIdx.x;
        const float x[kIn] = {f.a, f.th, f.log_r, 0.0f, 0.0f};
        float u[kIn];
        normalise(x, u);
        const float* b = Bm + j * kIn;
        const float c = fmaf(b[2], u[2], fmaf(b[1], u[1], b[0] * u[0]));
        f.proj[j] = make_float4(c, b[3], b[4], 0.0f);
    }
    for (int k = threadIdx.x; k < kCurveSamples; k += blockDim.x) {
        double al, be;
        const bool ok = critical_point(d.a, d.r_obs, d.theta_obs, static_cast<double>(k) / (kCurveSamples - 1), &al, &be);
        sa[k] = ok ? static_cast<float>(al) : nanf("");
        sbt[k] = ok ? static_cast<float>(be) : nanf("");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float mn = 1e30f, mx = -1e30f;
        int any = 0;
        for (int k = 0; k < kCurveSamples; ++k)
            if (sa[k] == sa[k]) {
                mn = fminf(mn, sa[k]);
                mx = fmaxf(mx, sa[k]);
                any = 1;
            }
        s_min = mn;
        s_max = mx;
        s_any = any;
    }
    __syncthreads();
    const float ac = 0.5f * (s_min + s_max);
    // psi and rho of the samples (in place)
    for (int k = threadIdx.x; k < kCurveSamples; k += blockDim.x) {
        const float da = sa[k] - ac, b = sbt[k];
        sa[k] = atan2f(b, da);  // NaN stays NaN
        sbt[k] = sqrtf(da * da + b * b);
    }
    __syncthreads();
    for (int j = threadIdx.x; j < kCurveBins; j += blockDim.x) {
        const float psi = 3.14159265f * (j + 0.5f) / kCurveBins;
        float rho = -1.0f, best = 1e30f, near_rho = -1.0f;
        for (int k = 0; k + 1 < kCurveSamples; ++k) {
            const float p0 = sa[k], p1 = sa[k + 1];
            if (!(p0 == p0) || !(p1 == p1)) continue;
            if ((psi - p0) * (psi - p1) <= 0.0f && p0 != p1) {
                const float t = (psi - p0) / (p1 - p0);
                rho = sbt[k] + t * (sbt[k + 1] - sbt[k]);
                break;
            }
            const float dd = fabsf(psi - p0);
            if (dd < best) {
                best = dd;
                near_rho = sbt[k];
            }
        }
        f.rho[j] = rho > 0.0f ? rho : near_rho;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < kCurveBins; j += blockDim.x) {
        const int jm = j > 0 ? j - 1 : 0, jp = j + 1 < kCurveBins ? j + 1 : kCurveBins - 1;
        const float dpsi = 3.14159265f * (jp - jm) / kCurveBins;
        const float drho = (f.rho[jp] - f.rho[jm]) / dpsi, r = f.rho[j];
        f.kn[j] = r > 0.0f ? r / sqrtf(r * r + drho * drho) : 1.0f;
    }
    if (threadIdx.x == 0) {
        f.alpha_c = ac;
        f.curve_ok = s_any;
    }
}

constexpr int kInfStages = 3;               // weight ring: 3 chunks in flight
constexpr int kTileRays = 128;
constexpr int kChunkBytes = 128 * 64 * 2;  // 16 KB: 128 rows x 64 BF16 of activations
constexpr int kHeadChunkBytes = 16 * 64 * 2;
// Epilogue warps per CTA (after the TMA and MMA warps): 16 at width 256 (two tile slots of 8: 4 TMEM lane
// quadrants x 2 column halves), 28 at width 64 (seven slots of 4 warps, one per lane quadrant; 960
// threads -- eight slots would pass the 1,024-thread limit of a block).
template <int HID>
__host__ __device__ constexpr int inf_epi_warps() { return HID == 64 ? 28 : 16; }
template <int HID>
__host__ __device__ constexpr int inf_threads() { return 64 + 32 * inf_epi_warps<HID>(); }
constexpr int kInfBars = 32;  // 64-bit mbarrier words reserved in shared memory
constexpr int kInfMisc = 8 * kInfBars + 16;  // barriers, TMEM slot and abort flag
// Per hidden width HID: one tile's activations (HID / 64 chunks of 64 columns), one weight chunk (all
// HID output rows x 64 K of a hidden layer), the shared memory of the kernel.
template <int HID>
__host__ __device__ constexpr int act_bytes() { return (HID / 64) * kChunkBytes; }
template <int HID>
__host__ __device__ constexpr int wchunk_bytes() { return HID * 64 * 2; }
// Tiles in flight per CTA: 2 at width 256 (2 x 256 TMEM columns, 8 epilogue warps each), 7 at width 64
// (7 x 64 of the 512 columns, 4 epilogue warps each -- one per TMEM lane quadrant -- at 64 registers a
// thread; six tiles at 72 registers ran 1.2 % slower, four at 96 registers 12 % slower). The epilogue can
// also serve several tiles per warp group in turn; at width 64 eight tiles that way measured slower.
template <int HID>
__host__ __device__ constexpr int inf_slots() { return HID == 64 ? 7 : 2; }
// At width 64 the whole network's weights (4 x 8 KB + the head's 2 KB) stay resident in shared memory,
// loaded once per CTA, and the MMA issuer serves whichever tile is ready; at width 256 they stream
// through a ring of kInfStages chunks in the MMA's order.
template <int HID>
__host__ __device__ constexpr bool inf_resident() { return HID == 64; }
template <int HID>
__host__ __device__ constexpr int inf_ring_bytes() {
    return inf_resident<HID>() ? kLayers * wchunk_bytes<HID>() : kInfStages * wchunk_bytes<HID>();
}
// (Resident weights) the biases as one more K slice of every layer's MMAs: a [128 x 64] tile whose first
// three columns are ones, and per layer a weight-layout tile whose first three columns hold the bias split
// into three BF16 parts (hi + mid + lo = the FP32 bias), the head's 16 rows last.
template <int HID>
__host__ __device__ constexpr int inf_bias_bytes() {
    return inf_resident<HID>() ? kChunkBytes + 4 * wchunk_bytes<HID>() + kHeadChunkBytes : 0;
}
template <int HID>
__host__ __device__ constexpr int inf_smem() {
    return inf_slots<HID>() * act_bytes<HID>() + inf_ring_bytes<HID>() + inf_bias_bytes<HID>() + 1024 + kInfMisc;
}

// Weight chunks per layer: 64-wide K slices of all output rows (N = HID per MMA; the head N = 16).
template <int HID>
__host__ __device__ constexpr int layer_chunks(int l) { return l == 0 ? 1 : HID / 64; }

struct InferArgs {
    const SurFrame* frames;
    int nframes;
    long long n;
    const float* bias[kLayers];
    const float* half_bias;  // [4][HID]: the hidden layers' biases halved
    uint8_t* outcome;
    double *r_disk, *phi_disk, *g, *theta_inf, *phi_inf;
    int32_t *steps, *rejected;
    int32_t* list;
    unsigned long long* n_list;
    float p_min, band;
    int* err;
    int accept;  // BHK_ACCEPT_*: which of the network's classes it may answer
};

// Byte offset of (row, col) in a 128-row x 64-column BF16 tile with the 128-byte swizzle.
__device__ __forceinline__ uint32_t sw128(int row, int col) {
    return static_cast<uint32_t>(row * 128 + ((((col >> 3) ^ (row & 7))) << 4) + ((col & 7) << 1));
}

// Stores 16 BF16 (8 packed words) of `row` at columns c0 .. c0+15 of the 256-wide activation.
__device__ __forceinline__ void store_act16(uint8_t* act, int row, int c0, const uint32_t* w) {
    uint8_t* chunk = act + (c0 >> 6) * kChunkBytes;
    const int c = c0 & 63;
    *reinterpret_cast<uint4*>(chunk + sw128(row, c)) = make_uint4(w[0], w[1], w[2], w[3]);
    *reinterpret_cast<uint4*>(chunk + sw128(row, c + 8)) = make_uint4(w[4], w[5], w[6], w[7]);
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    uint32_t r;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    return r;
}

// SiLU of 32 accumulator columns that already hold z / 2 (raw FP32 bits) -> 16 packed BF16x2 words.
__device__ __forceinline__ void silu32_half(const uint32_t (&v)[32], uint32_t (&w)[16]) {
#pragma unroll
    for (int q = 0; q < 16; ++q) w[q] = silu2_half(__uint_as_float(v[2 * q]), __uint_as_float(v[2 * q + 1]));
}

// SiLU of 32 accumulator columns (raw FP32 bits) with halved biases hb -> 16 packed BF16x2 words.
__device__ __forceinline__ void silu32(const uint32_t (&v)[32], const float* hb, uint32_t (&w)[16]) {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const float4 b = __ldg(reinterpret_cast<const float4*>(hb) + q);
        w[2 * q] = silu2_half(fmaf(__uint_as_float(v[4 * q]), 0.5f, b.x), fmaf(__uint_as_float(v[4 * q + 1]), 0.5f, b.y));
        w[2 * q + 1] =
            silu2_half(fmaf(__uint_as_float(v[4 * q + 2]), 0.5f, b.z), fmaf(__uint_as_float(v[4 * q + 3]), 0.5f, b.w));
    }
}

// NS = inf_slots<HID>() tiles in flight per CTA: while the tensor core runs one tile's layer, the other
// tiles' epilogue warps turn their accumulators into the next layer's operand. Each tile slot owns HID
// TMEM columns and an activation buffer of HID columns; the weight ring is shared and filled in the
// MMA's order (group of NS tiles, layer, slot, chunk). Every MMA is 128 x HID x 16, so each activation
// slice is read from shared memory once per layer. CTA b takes tiles b, b + grid, ...
template <int HID>
__global__ void __launch_bounds__(inf_threads<HID>(), 1)
infer_kernel(const __grid_constant__ CUtensorMap tW0, const __grid_constant__ CUtensorMap tW1,
             const __grid_constant__ CUtensorMap tW2, const __grid_constant__ CUtensorMap tW3,
             const __grid_constant__ CUtensorMap tW4, InferArgs ia) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    constexpr int NS = inf_slots<HID>();
    constexpr int kActBytes = act_bytes<HID>(), kWChunkBytes = wchunk_bytes<HID>();
    constexpr uint32_t kTmemCols = NS * HID <= 256 ? 256 : 512;  // NS tile slots of HID columns (a power of 2)
    // A tile's epilogue: 4 warps (one per TMEM lane quadrant) at width 64, 8 (two column halves) at 256.
    constexpr int kHalves = HID == 64 ? 1 : 2, kWarpsPerSlot = 4 * kHalves;
    constexpr int kEpiWarps = inf_epi_warps<HID>();
    static_assert(kEpiWarps % kWarpsPerSlot == 0 && NS % (kEpiWarps / kWarpsPerSlot) == 0, "slot mapping");
    static_assert(kInfStages + kInfStages + 2 * NS + 1 <= kInfBars, "the mbarriers fit their words");
    constexpr bool kResident = inf_resident<HID>();
    uint8_t* ring = base + NS * kActBytes;  // the weight ring, or (kResident) layer l's weights at l chunks
    uint8_t* sOnes = ring + inf_ring_bytes<HID>();  // (kResident) the ones tile, then the bias tiles
    uint8_t* sBiasT = sOnes + kChunkBytes;
    uint64_t* full = reinterpret_cast<uint64_t*>(sOnes + inf_bias_bytes<HID>());
    uint64_t* empty = full + kInfStages;
    uint64_t* act_ready = empty + kInfStages;  // [NS]
    uint64_t* acc_full = act_ready + NS;       // [NS]
    uint64_t* drain = acc_full + NS;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(full + kInfBars);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long ntiles = (ia.n + kTileRays - 1) / kTileRays;
    const long long cid = blockIdx.x, ncl = gridDim.x;
    const long long n_my = cid < ntiles ? (ntiles - cid + ncl - 1) / ncl : 0;
    const long long groups = (n_my + NS - 1) / NS;
    if (threadIdx.x == 0) {
        for (int st = 0; st < kInfStages; ++st) {
            tc::mbar_init(&full[st], 1);
            tc::mbar_init(&empty[st], 1);
        }
        for (int sl = 0; sl < NS; ++sl) {
            tc::mbar_init(&act_ready[sl], kWarpsPerSlot);  // one arrival per warp
            tc::mbar_init(&acc_full[sl], 1);
        }
        tc::mbar_init(drain, 1);
        *abort_flag = 0;
        tc::fence_mbar_init();
        tc::prefetch_tmap(&tW0);
        tc::prefetch_tmap(&tW1);
        tc::prefetch_tmap(&tW2);
        tc::prefetch_tmap(&tW3);
        tc::prefetch_tmap(&tW4);
    }
    if (warp == 1) tc::tmem_alloc(tmem_slot, kTmemCols);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    auto give_up = [&]() {
        *abort_flag = 1;
        atomicExch(ia.err, 1);
    };

    if constexpr (kResident) {
        // ---- the network's weights, once, prepared by all threads: the hidden layers' halved (exact), so
        // that the accumulators hold z / 2, the SiLU's argument; the biases (halved for the hidden layers)
        // as the MMA chain's last K slice against the ones tile.
        if (n_my > 0) {
            if (threadIdx.x == 0) {
                tc::mbar_expect_tx(&full[0], 4 * kWChunkBytes + kHeadChunkBytes);
                tc::tma_load_2d(ring + 0 * kWChunkBytes, &tW0, 0, 0, &full[0]);
                tc::tma_load_2d(ring + 1 * kWChunkBytes, &tW1, 0, 0, &full[0]);
                tc::tma_load_2d(ring + 2 * kWChunkBytes, &tW2, 0, 0, &full[0]);
                tc::tma_load_2d(ring + 3 * kWChunkBytes, &tW3, 0, 0, &full[0]);
                tc::tma_load_2d(ring + 4 * kWChunkBytes, &tW4, 0, 0, &full[0]);
            }
            for (int i = threadIdx.x; i < kTileRays * 2; i += blockDim.x) {  // columns 0-7 and 8-15 of each row
                const int r = i >> 1, h = i & 1;
                *reinterpret_cast<uint4*>(sOnes + sw128(r, 8 * h)) =
                    h == 0 ? make_uint4(0x3F803F80u, 0x00003F80u, 0u, 0u) : make_uint4(0u, 0u, 0u, 0u);
            }
            for (int i = threadIdx.x; i < 4 * HID + 16; i += blockDim.x) {
                const int l = i < 4 * HID ? i / HID : 4, n = i < 4 * HID ? i % HID : i - 4 * HID;
                const float b = l < 4 ? 0.5f * ia.bias[l][n] : (n < kOut ? ia.bias[4][n] : 0.0f);
                const bf16 hi = __float2bfloat16_rn(b);
                const float r1 = b - __bfloat162float(hi);
                const bf16 mid = __float2bfloat16_rn(r1);
                const bf16 lo = __float2bfloat16_rn(r1 - __bfloat162float(mid));
                uint8_t* t = sBiasT + l * kWChunkBytes;
                *reinterpret_cast<uint4*>(t + sw128(n, 0)) =
                    make_uint4(static_cast<uint32_t>(__bfloat16_as_ushort(hi)) |
                                   (static_cast<uint32_t>(__bfloat16_as_ushort(mid)) << 16),
                               static_cast<uint32_t>(__bfloat16_as_ushort(lo)), 0u, 0u);
                *reinterpret_cast<uint4*>(t + sw128(n, 8)) = make_uint4(0u, 0u, 0u, 0u);
            }
            if (!tc::mbar_wait(&full[0], 0)) {  // landed (bounded)
                if (threadIdx.x == 0) give_up();
            } else {
                uint32_t* w = reinterpret_cast<uint32_t*>(ring);
                for (int i = threadIdx.x; i < 4 * kWChunkBytes / 4; i += blockDim.x) {
                    uint32_t h;
                    asm("mul.rn.bf16x2 %0, %1, %2;" : "=r"(h) : "r"(w[i]), "r"(0x3F003F00u));
                    w[i] = h;
                }
            }
            tc::fence_proxy_async();  // the generic-proxy writes, before the tensor core reads them
        }
        __syncthreads();
    }

    if (warp == 0 && kResident) {
        // (the weights were loaded above)
    } else if (warp == 1 && kResident) {
        if (lane == 0) {  // ---- MMA issuer: whichever tile slot has its next layer's input ready
            constexpr uint32_t kIdHid = tc::idesc_bf16(128, HID), kId16 = tc::idesc_bf16(128, 16);
            uint32_t act_n[NS] = {};
            int layer[NS] = {};
            long long left[NS];
            long long total = 0;
            for (int sl = 0; sl < NS; ++sl) {
                const long long tiles = sl < n_my ? (n_my - sl + NS - 1) / NS : 0;
                left[sl] = tiles * kLayers;
                total += left[sl];
            }
            bool ok = total == 0 || tc::mbar_wait(&full[0], 0);
            if (!ok) give_up();
            tc::fence_after_sync();
            const uint64_t ones_d = tc::smem_desc_sw128(sOnes);
            uint32_t idle = 0;  // sweeps without progress (bounded)
            while (ok && total > 0) {
                bool progress = false;
                for (int sl = 0; sl < NS; ++sl) {
                    if (left[sl] == 0 || !tc::mbar_test(&act_ready[sl], act_n[sl] & 1)) continue;
                    ++act_n[sl];
                    tc::fence_after_sync();
                    const int l = layer[sl];
                    const uint64_t ad = tc::smem_desc_sw128(base + sl * kActBytes);
                    const uint64_t bd = tc::smem_desc_sw128(ring + l * kWChunkBytes);
                    const uint32_t d = tmem + static_cast<uint32_t>(HID * sl);
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk)
                        tc::mma_bf16(d, ad + 2 * kk, bd + 2 * kk, l < 4 ? kIdHid : kId16, kk ? 1u : 0u);
                    tc::mma_bf16(d, ones_d, tc::smem_desc_sw128(sBiasT + l * kWChunkBytes), l < 4 ? kIdHid : kId16, 1u);
                    tc::mma_commit(&acc_full[sl]);
                    layer[sl] = l + 1 == kLayers ? 0 : l + 1;
                    --left[sl];
                    --total;
                    progress = true;
                }
                if (progress) {
                    idle = 0;
                } else if (++idle > tc::kSpinLimit || *abort_flag) {
                    if (!*abort_flag) give_up();
                    ok = false;
                }
            }
            // All MMAs issued have finished before TMEM is released (bounded).
            tc::mma_commit(drain);
            tc::mbar_wait(drain, 0);
        }
    } else if (warp == 0) {
        if (lane == 0) {  // ---- TMA producer, in the MMA's order
            long long q = 0;
            bool ok = true;
            for (long long p = 0; p < groups && ok; ++p)
                for (int l = 0; l < kLayers && ok; ++l)
                    for (int sl = 0; sl < NS && ok; ++sl) {
                        if (NS * p + sl >= n_my) continue;
                        for (int c = 0; c < layer_chunks<HID>(l); ++c, ++q) {
                            if (*abort_flag) { ok = false; break; }
                            const int st = static_cast<int>(q % kInfStages);
                            const long long j = q / kInfStages;
                            if (j > 0 && !tc::mbar_wait(&empty[st], static_cast<uint32_t>((j - 1) & 1))) {
                                give_up();
                                ok = false;
                                break;
                            }
                            const int kc = c;
                            const CUtensorMap* m = l == 0 ? &tW0 : l == 1 ? &tW1 : l == 2 ? &tW2 : l == 3 ? &tW3 : &tW4;
                            tc::mbar_expect_tx(&full[st], l < 4 ? kWChunkBytes : kHeadChunkBytes);
                            tc::tma_load_2d(ring + st * kWChunkBytes, m, kc * 64, 0, &full[st]);
                        }
                    }
            // Before the CTA may exit (bounded): every load of the last ring round has landed.
            for (long long r = q - kInfStages; r < q; ++r)
                if (r >= 0) tc::mbar_wait(&full[r % kInfStages], static_cast<uint32_t>((r / kInfStages) & 1));
        }
    } else if (warp == 1) {
        if (lane == 0) {  // ---- MMA issuer
            constexpr uint32_t kIdHid = tc::idesc_bf16(128, HID), kId16 = tc::idesc_bf16(128, 16);
            long long q = 0;
            uint32_t act_n[NS] = {};
            bool ok = true;
            for (long long p = 0; p < groups && ok; ++p)
                for (int l = 0; l < kLayers && ok; ++l)
                    for (int sl = 0; sl < NS && ok; ++sl) {
                        if (NS * p + sl >= n_my) continue;
                        if (*abort_flag || !tc::mbar_wait(&act_ready[sl], act_n[sl] & 1)) {
                            if (!*abort_flag) give_up();
                            ok = false;
                            break;
                        }
                        ++act_n[sl];
                        tc::fence_after_sync();
                        uint8_t* act = base + sl * kActBytes;
                        for (int c = 0; c < layer_chunks<HID>(l); ++c, ++q) {
                            const int st = static_cast<int>(q % kInfStages);
                            if (!tc::mbar_wait(&full[st], static_cast<uint32_t>((q / kInfStages) & 1))) {
                                give_up();
                                ok = false;
                                break;
                            }
                            tc::fence_after_sync();
                            const int kc = c;
                            const uint64_t ad = tc::smem_desc_sw128(act + kc * kChunkBytes);
                            const uint64_t bd = tc::smem_desc_sw128(ring + st * kWChunkBytes);
                            const uint32_t d = tmem + static_cast<uint32_t>(HID * sl);
#pragma unroll
                            for (int kk = 0; kk < 4; ++kk)
                                tc::mma_bf16(d, ad + 2 * kk, bd + 2 * kk, l < 4 ? kIdHid : kId16, (kc | kk) ? 1u : 0u);
                            tc::mma_commit(&empty[st]);
                        }
                        if (ok) tc::mma_commit(&acc_full[sl]);
                    }
            // All MMAs issued have finished before TMEM is released (bounded).
            tc::mma_commit(drain);
            tc::mbar_wait(drain, 0);
        }
    } else {  // ---- warps 2..17: features, epilogues, decode (thread = ray of its slot's tile)
        // kGroupsE warp groups of kWarpsPerSlot warps; group g serves the TPW slots g, g + kGroupsE, ...,
        // one phase of each in turn (features, the four hidden epilogues, the head), so that one tile's
        // MMA runs while the group works on its other tile.
        constexpr int kGroupsE = kEpiWarps / kWarpsPerSlot, TPW = NS / kGroupsE;
        const int ew = warp - 2;
        const int grp = ew / kWarpsPerSlot;
        const int half = (ew >> 2) % kHalves;  // its share of the columns (and of the 32 frequencies)
        const int q4 = warp & 3;               // TMEM lane quadrant this warp may access
        const int row = 32 * q4 + lane;
        uint32_t acc_n[TPW] = {};
        // Every exit decision is taken by the whole warp (the TMEM loads and the list append are
        // warp-collective).
        bool ok = true;
        for (long long it = 0; ok; ++it) {
            if (grp + NS * it >= n_my) break;  // (slot grp has the most tiles of this group's slots)
            if (__any_sync(0xffffffffu, *abort_flag)) break;
            bool has[TPW], live[TPW];
            long long ray[TPW];
            int fi[TPW];
            float alpha[TPW], beta[TPW];
#pragma unroll
            for (int v = 0; v < TPW; ++v) {  // ---- features
                const int slot = grp + kGroupsE * v;
                has[v] = slot + NS * it < n_my;
                ray[v] = (cid + (slot + NS * it) * ncl) * kTileRays + row;
                live[v] = has[v] && ray[v] < ia.n;
                fi[v] = 0;
                alpha[v] = beta[v] = 0.0f;
                if (!has[v]) continue;
                uint8_t* act = base + slot * kActBytes;
                constexpr int kFreqPer = kFreq / kHalves;  // frequencies of this thread, in blocks of 16
                float u[kIn] = {};
                if (live[v]) {
                    int lo = 0, hi = ia.nframes - 1;
                    while (lo < hi) {
                        const int mid = (lo + hi + 1) >> 1;
                        if (ia.frames[mid].offset <= ray[v]) lo = mid; else hi = mid - 1;
                    }
                    fi[v] = lo;
                    const SurFrame& f = ia.frames[lo];
                    const int local = static_cast<int>(ray[v] - f.offset);
                    const int pr = local / f.width, pc = local - pr * f.width;
                    alpha[v] = static_cast<float>(f.alpha_lo + (pc + 0.5) * f.px);
                    beta[v] = static_cast<float>(f.beta_hi - (pr + 0.5) * f.py);
                    const float x[kIn] = {f.a, f.th, f.log_r, alpha[v], beta[v]};
                    normalise(x, u);
                }
#pragma unroll
                for (int fb = 0; fb < kFreqPer / 16; ++fb) {
                    const int j0 = kFreqPer * half + 16 * fb;  // first frequency of this block
                    uint32_t fs[8], fc[8];  // the block's 16 sines and 16 cosines, packed
                    if (live[v]) {
#pragma unroll
                        for (int j = 0; j < 16; j += 2) {
                            float sv[2], cv[2];
#pragma unroll
                            for (int e = 0; e < 2; ++e) {
                                const float4 pj = ia.frames[fi[v]].proj[j0 + j + e];
                                const float pp = fmaf(pj.z, u[4], fmaf(pj.y, u[3], pj.x));
                                __sincosf(6.28318530717958648f * (pp - rintf(pp)), &sv[e], &cv[e]);
                            }
                            fs[j >> 1] = pack_bf16(sv[0], sv[1]);
                            fc[j >> 1] = pack_bf16(cv[0], cv[1]);
                        }
                    } else {
#pragma unroll
                        for (int j = 0; j < 8; ++j) fs[j] = fc[j] = 0u;
                    }
                    store_act16(act, row, j0, fs);
                    store_act16(act, row, kFreq + j0, fc);
                }
                // Every lane's activations are visible to the tensor core before its warp's one arrival.
                tc::fence_proxy_async();
                tc::fence_before_sync();
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(&act_ready[slot]);
            }
            for (int l = 0; l < 4 && ok; ++l) {  // ---- hidden layers
#pragma unroll
                for (int v = 0; v < TPW; ++v) {
                    if (!has[v] || !ok) continue;
                    const int slot = grp + kGroupsE * v;
                    if (!__all_sync(0xffffffffu, tc::mbar_wait(&acc_full[slot], acc_n[v] & 1))) {
                        if (lane == 0) give_up();
                        ok = false;
                        continue;
                    }
                    ++acc_n[v];
                    tc::fence_after_sync();
                    uint8_t* act = base + slot * kActBytes;
                    const uint32_t trow =
                        tmem + (static_cast<uint32_t>(32 * q4) << 16) + static_cast<uint32_t>(HID) * slot;
                    constexpr int kHalf = HID / kHalves, kGroups = kHalf / 32;  // this warp's columns, in 32s
                    const float* hb = ia.half_bias + l * HID + kHalf * half;
                    const uint32_t cb = trow + static_cast<uint32_t>(kHalf) * half;
                    if constexpr (kResident) {  // 32 columns at a time (the register budget of 28 warps)
                        static_assert(HID == 64, "resident weights at width 64");
                        uint32_t ra[32];
#pragma unroll 1
                        for (int jj = 0; jj < kGroups; ++jj) {
                            tc::tmem_ld32_issue(cb + 32u * jj, ra);
                            tc::tmem_wait32(ra);
                            uint32_t w[16];
                            silu32_half(ra, w);  // the accumulator holds z / 2, bias included
                            store_act16(act, row, kHalf * half + 32 * jj, w);
                            store_act16(act, row, kHalf * half + 32 * jj + 16, w + 8);
                        }
                    } else {  // the next 32 columns' load in flight while the current ones are processed
                        uint32_t ra[32], rb[32];
                        tc::tmem_ld32_issue(cb, ra);
                        tc::tmem_wait32(ra);
#pragma unroll
                        for (int jj = 0; jj < kGroups; ++jj) {
                            uint32_t(&cur)[32] = (jj & 1) ? rb : ra;
                            uint32_t(&nxt)[32] = (jj & 1) ? ra : rb;
                            if (jj + 1 < kGroups) tc::tmem_ld32_issue(cb + 32u * (jj + 1), nxt);
                            uint32_t w[16];
                            silu32(cur, hb + 32 * jj, w);
                            store_act16(act, row, kHalf * half + 32 * jj, w);
                            store_act16(act, row, kHalf * half + 32 * jj + 16, w + 8);
                            if (jj + 1 < kGroups) tc::tmem_wait32(nxt);
                        }
                    }
                    tc::fence_proxy_async();
                    tc::fence_before_sync();
                    __syncwarp();
                    if (lane == 0) tc::mbar_arrive(&act_ready[slot]);
                }
            }
            if (!ok) break;
#pragma unroll
            for (int v = 0; v < TPW; ++v) {  // ---- the head: decode and the fallback decision
                if (!has[v] || !ok) continue;
                const int slot = grp + kGroupsE * v;
                if (!__all_sync(0xffffffffu, tc::mbar_wait(&acc_full[slot], acc_n[v] & 1))) {
                    if (lane == 0) give_up();
                    ok = false;
                    continue;
                }
                ++acc_n[v];
                tc::fence_after_sync();
                if (half == 1) {
                    tc::fence_before_sync();
                    continue;  // the head's 8 outputs are decoded by the first half
                }
                const uint32_t trow =
                    tmem + (static_cast<uint32_t>(32 * q4) << 16) + static_cast<uint32_t>(HID) * slot;
                float y[16];
                tc::tmem_ld16(trow, y);
                tc::fence_before_sync();
                bool fb = false;
                if (live[v]) {
                    if constexpr (!kResident) {  // (resident weights: the MMAs added the bias)
                        const float* b4 = ia.bias[4];
#pragma unroll
                        for (int i = 0; i < kOut; ++i) y[i] += __ldg(b4 + i);
                    }
                    int cls = 0;
                    float mx = y[0];
                    if (y[1] > mx) { mx = y[1]; cls = 1; }
                    if (y[2] > mx) { mx = y[2]; cls = 2; }
                    const float zsum = __expf(y[0] - mx) + __expf(y[1] - mx) + __expf(y[2] - mx);
                    const float pmax = 1.0f / zsum;
                    const double nan = __longlong_as_double(0x7ff8000000000000ll);
                    double rd = nan, gg = nan, ti = nan, pi = nan;
                    if (cls == 1) {
                        rd = 30.0 * y[3];
                        gg = __expf(y[4]);
                    } else if (cls == 2) {
                        const float nrm = sqrtf(y[5] * y[5] + y[6] * y[6] + y[7] * y[7]);
                        const float dz = fminf(1.0f, fmaxf(-1.0f, y[7] / nrm));
                        ti = acosf(dz);
                        pi = atan2f(y[6], y[5]);
                    }
                    const SurFrame& f = ia.frames[fi[v]];
                    bool band = false;
                    if (f.curve_ok) {
                        const float da = alpha[v] - f.alpha_c, ab_ = fabsf(beta[v]);
                        const float psi = atan2f(ab_, da);
                        const int jb = min(kCurveBins - 1, max(0, static_cast<int>(psi * (kCurveBins / 3.14159265f))));
                        band = fabsf(sqrtf(da * da + ab_ * ab_) - f.rho[jb]) * f.kn[jb] < ia.band;
                    }
                    // Answers limited to captured rays carry no continuous output, so where the class
                    // is right they are exactly the tracer's (the network's r_disk, g and direction
                    // are not used).
                    fb = pmax < ia.p_min || band || fabsf(alpha[v]) < f.snap || !(zsum == zsum) ||
                         (ia.accept == BHK_ACCEPT_CAPTURED && cls != 0);
                    const long long r = ray[v];
                    ia.outcome[r] = static_cast<uint8_t>(cls + 1);
                    if (ia.r_disk) ia.r_disk[r] = rd;
                    if (ia.phi_disk) ia.phi_disk[r] = nan;
                    if (ia.g) ia.g[r] = gg;
                    if (ia.theta_inf) ia.theta_inf[r] = ti;
                    if (ia.phi_inf) ia.phi_inf[r] = pi;
                    if (ia.steps) ia.steps[r] = 0;
                    if (ia.rejected) ia.rejected[r] = 0;
                }
                const unsigned m = __ballot_sync(0xffffffffu, fb);
                if (m) {
                    unsigned long long b0 = 0;
                    if (lane == 0) b0 = atomicAdd(ia.n_list, static_cast<unsigned long long>(__popc(m)));
                    b0 = __shfl_sync(0xffffffffu, b0, 0);
                    if (fb) ia.list[b0 + __popc(m & ((1u << lane) - 1u))] = static_cast<int32_t>(ray[v]);
                }
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 1) tc::tmem_dealloc(tmem, kTmemCols);
}

__global__ void halve_bias_kernel(const float* b0, const float* b1, const float* b2, const float* b3, float* out) {
    const float* b = blockIdx.x == 0 ? b0 : blockIdx.x == 1 ? b1 : blockIdx.x == 2 ? b2 : b3;
    out[blockIdx.x * blockDim.x + threadIdx.x] = 0.5f * b[threadIdx.x];  // blockDim.x = the hidden width
}

// Copies compact fallback results (entry i = pixel list[i]) into the full-image outputs.
__global__ void scatter_kernel(const int32_t* __restrict__ list, long long n, bhk_rays_out src, bhk_rays_out dst) {
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long p = list[i];
        if (dst.outcome) dst.outcome[p] = src.outcome[i];
        if (dst.r_disk) dst.r_disk[p] = src.r_disk[i];
        if (dst.phi_disk) dst.phi_disk[p] = src.phi_disk[i];
        if (dst.g) dst.g[p] = src.g[i];
        if (dst.theta_inf) dst.theta_inf[p] = src.theta_inf[i];
        if (dst.phi_inf) dst.phi_inf[p] = src.phi_inf[i];
        if (dst.steps) dst.steps[p] = src.steps[i];
        if (dst.rejected) dst.rejected[p] = src.rejected[i];
    }
}

}  // namespace sur
}  // namespace bhk

extern "C" bhk_status bhk_surrogate_render(bhk_surrogate* s, bhk_context* ctx, const bhk_frame_desc* frames,
                                           int32_t nframes, const bhk_trace_opts* opts,
                                           const bhk_render_opts* ropts, const bhk_rays_out* out,
                                           bhk_render_stats* stats, void* stream) {
    using namespace bhk::sur;
    if (!s || !ctx || !frames || nframes <= 0 || !out || !out->outcome) {
        set_last_error("bhk_surrogate_render: null argument (outcome output required)");
        return BHK_EINVAL;
    }
    long long total = 0;
    for (int i = 0; i < nframes; ++i) {
        const bhk_frame_desc& d = frames[i];
        if (d.width <= 0 || d.height <= 0 || !(std::fabs(d.a) < 1.0) || !(d.theta_obs > 0.0 && d.theta_obs < M_PI) ||
            !(d.r_obs > 1.0 + std::sqrt(1.0 - d.a * d.a)) || !(d.r_disk_out >= 0.0)) {
            set_last_error("bhk_surrogate_render: invalid frame");
            return BHK_EINVAL;
        }
        total += static_cast<long long>(d.width) * d.height;
    }
    if (total > (1ll << 31) - 1) {
        set_last_error("bhk_surrogate_render: more than 2^31 - 1 rays in one call");
        return BHK_EINVAL;
    }
    bhk_render_opts ro{};
    ro.p_min = 0.99;
    ro.band = 0.05;
    ro.fallback = 1;
    if (ropts) ro = *ropts;
    if (ro.accept != BHK_ACCEPT_ALL && ro.accept != BHK_ACCEPT_CAPTURED) {
        set_last_error("bhk_surrogate_render: accept must be BHK_ACCEPT_ALL or BHK_ACCEPT_CAPTURED");
        return BHK_EINVAL;
    }
    std::lock_guard<std::mutex> lock_ctx(bhk::context_mutex(ctx));
    std::lock_guard<std::mutex> lock(s->mu);
    if (cudaSetDevice(s->device) != cudaSuccess || bhk::context_device(ctx) != s->device) {
        set_last_error("bhk_surrogate_render: surrogate and context must share the device");
        return BHK_EINVAL;
    }
    cudaStream_t st = bhk::context_stream(ctx, stream);
    // scratch
    auto fail_cuda = [](cudaError_t e, const char* what) {
        set_last_error(std::string("bhk_surrogate_render: ") + what + ": " + cudaGetErrorString(e));
        return BHK_ECUDA;
    };
    cudaError_t e = cudaSuccess;
    const size_t fbytes = sizeof(SurFrame) * nframes + sizeof(bhk_frame_desc) * nframes;
    if (fbytes > s->cap_frames) {
        if (s->frames_dev) cudaFree(s->frames_dev);
        s->frames_dev = nullptr;
        e = cudaMalloc(&s->frames_dev, fbytes);
        s->cap_frames = e == cudaSuccess ? fbytes : 0;
        if (e != cudaSuccess) return fail_cuda(e, "frame table");
    }
    if (static_cast<size_t>(total) > s->cap_list) {
        if (s->list) cudaFree(s->list);
        s->list = nullptr;
        e = cudaMalloc(reinterpret_cast<void**>(&s->list), sizeof(int32_t) * total);
        s->cap_list = e == cudaSuccess ? static_cast<size_t>(total) : 0;
        if (e != cudaSuccess) return fail_cuda(e, "fallback list");
    }
    std::vector<SurFrame> hf(nframes);
    long long off = 0;
    for (int i = 0; i < nframes; ++i) {
        const bhk_frame_desc& d = frames[i];
        SurFrame& f = hf[i];
        std::memset(static_cast<void*>(&f), 0, sizeof(SurFrame));
        f.alpha_lo = d.alpha_lo;
        f.beta_hi = d.beta_hi;
        f.px = (d.alpha_hi - d.alpha_lo) / d.width;
        f.py = (d.beta_hi - d.beta_lo) / d.height;
        f.offset = off;
        f.width = d.width;
        f.height = d.height;
        f.a = static_cast<float>(d.a);
        f.th = static_cast<float>(d.theta_obs);
        f.log_r = static_cast<float>(std::log10(d.r_obs));
        // L = 0 snapping acts where |L| < 3e-4 sqrt(Q + a^2 E^2); with L ~ -alpha sin(theta) and
        // Q + a^2 E^2 below 40 M^2 inside the images this is |alpha| sin(theta) < 2e-3: widened 2x.
        f.snap = static_cast<float>(4e-3 / std::max(std::sin(d.theta_obs), 0.05));
        off += static_cast<long long>(d.width) * d.height;
    }
    SurFrame* dframes = static_cast<SurFrame*>(s->frames_dev);
    bhk_frame_desc* ddesc = reinterpret_cast<bhk_frame_desc*>(dframes + nframes);
    e = cudaMemcpyAsync(dframes, hf.data(), sizeof(SurFrame) * nframes, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ddesc, frames, sizeof(bhk_frame_desc) * nframes, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return fail_cuda(e, "frame upload");
    curve_table_kernel<<<nframes, 256, 0, st>>>(dframes, ddesc, s->Bm);
    const int H = s->hid;
    auto* kern = H == 64 ? &infer_kernel<64> : &infer_kernel<256>;
    const int smem = H == 64 ? inf_smem<64>() : inf_smem<256>();
    const int threads = H == 64 ? inf_threads<64>() : inf_threads<256>();
    static std::once_flag attr;
    std::call_once(attr, [] {
        cudaFuncSetAttribute(infer_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, inf_smem<64>());
        cudaFuncSetAttribute(infer_kernel<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, inf_smem<256>());
    });
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device);
    // The grid is the number of CTAs resident at once (the static tile schedule must not need a second
    // wave): one per SM at width 256 (its shared memory and all 512 TMEM columns), as many as fit at 64
    // (2 x 64 TMEM columns each).
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    const int resident = sms * std::min(per_sm, 4);
    Maps M;
    CUtensorMap w4;
    const uint32_t slice = static_cast<uint32_t>(H);
    if (!make_tmap(&M.W[0], s->w_rm[0], H, kFeat, slice) || !make_tmap(&M.W[1], s->w_rm[1], H, H, slice) ||
        !make_tmap(&M.W[2], s->w_rm[2], H, H, slice) || !make_tmap(&M.W[3], s->w_rm[3], H, H, slice) ||
        !make_tmap(&w4, s->w_rm[4], kOutPad, H, 16)) {
        set_last_error("bhk_surrogate_render: tensor map creation failed");
        return BHK_ECUDA;
    }
    const long long ntiles = (total + kTileRays - 1) / kTileRays;
    const int grid = static_cast<int>(std::min<long long>(ntiles, resident));
    halve_bias_kernel<<<4, H, 0, st>>>(s->p + s->L.b[0], s->p + s->L.b[1], s->p + s->L.b[2], s->p + s->L.b[3],
                                       s->half_bias);
    InferArgs ia{};
    ia.accept = ro.accept;
    ia.half_bias = s->half_bias;
    ia.frames = dframes;
    ia.nframes = nframes;
    ia.n = total;
    for (int l = 0; l < kLayers; ++l) ia.bias[l] = s->p + s->L.b[l];
    ia.outcome = out->outcome;
    ia.r_disk = out->r_disk;
    ia.phi_disk = out->phi_disk;
    ia.g = out->g;
    ia.theta_inf = out->theta_inf;
    ia.phi_inf = out->phi_inf;
    ia.steps = out->steps;
    ia.rejected = out->rejected;
    ia.list = s->list;
    ia.n_list = s->n_list;
    ia.p_min = static_cast<float>(ro.p_min);
    ia.band = static_cast<float>(ro.band);
    ia.err = s->err;
    e = cudaMemsetAsync(s->n_list, 0, sizeof(unsigned long long), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->err, 0, sizeof(int), st);
    if (e == cudaSuccess) e = cudaEventRecord(s->ev[0], st);
    if (e != cudaSuccess) return fail_cuda(e, "launch set-up");
    kern<<<grid, threads, smem, st>>>(M.W[0], M.W[1], M.W[2], M.W[3], w4, ia);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventRecord(s->ev[1], st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s->n_list_host, s->n_list, 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail_cuda(e, "inference");
    {
        int herr = 0;
        cudaMemcpy(&herr, s->err, sizeof(int), cudaMemcpyDeviceToHost);
        if (herr) {
            set_last_error("bhk_surrogate_render: a tensor-core pipeline wait timed out");
            return BHK_ECUDA;
        }
    }
    const long long nfb = static_cast<long long>(*s->n_list_host);
    double trace_ms = 0.0;
    bhk_status rs = BHK_OK;
    if (ro.fallback && nfb > 0) {
        bhk_rays_out used{};
        rs = bhk::trace_pixel_list(ctx, frames, nframes, s->list, nfb, opts, nullptr, &used, st);
        if (rs != BHK_OK) return rs;
        scatter_kernel<<<1024, 256, 0, st>>>(s->list, nfb, used, *out);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventRecord(s->ev[2], st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return fail_cuda(e, "fallback trace");
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, s->ev[1], s->ev[2]) == cudaSuccess) trace_ms = ms;
        else cudaGetLastError();
    }
    if (stats) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, s->ev[0], s->ev[1]) != cudaSuccess) {
            cudaGetLastError();
            ms = 0.0f;
        }
        stats->rays = total;
        stats->fallback = nfb;
        stats->infer_ms = ms;
        stats->trace_ms = trace_ms;
        stats->accept = ro.accept;
        stats->grid = grid;
    }
    return rs;
}

extern "C" bhk_status bhk_surrogate_fallback_list(bhk_surrogate* s, int32_t* dst, int64_t cap, int64_t* n) {
    if (!s || !n || cap < 0 || (cap > 0 && !dst)) return BHK_EINVAL;
    std::lock_guard<std::mutex> lock(s->mu);
    const int64_t have = s->n_list_host ? static_cast<int64_t>(*s->n_list_host) : 0;
    *n = have;
    const int64_t m = std::min(have, cap);
    if (m > 0) {
        cudaSetDevice(s->device);
        if (cudaMemcpy(dst, s->list, sizeof(int32_t) * m, cudaMemcpyDeviceToDevice) != cudaSuccess) {
            set_last_error("bhk_surrogate_fallback_list: copy failed");
            return BHK_ECUDA;
        }
    }
    return BHK_OK;
}

// ============================================================================ training set ====
//
// Rays drawn as the surrogate's training set specifies -- a uniform on [0, 0.998], theta_obs uniform
// on [5, 89] degrees, log10 r_obs uniform on [log10 20, 3], (alpha, beta) uniform in a disk of radius
// 1.5 x the shadow radius -- traced by the mixed tracer and turned into (inputs, classes, targets).
// The shadow radius (largest distance of the analytic critical curve from the image centre) comes
// from a table over (a, theta, log10 r) built on the device and interpolated trilinearly.

namespace bhk {
namespace sur {

constexpr int kTabA = 24, kTabT = 24, kTabR = 12, kTabSamples = 512;
constexpr double kAMax = 0.998, kThLo = 5.0 * kPi / 180.0, kThHi = 89.0 * kPi / 180.0;
constexpr double kLogRLo = 1.3010299956639813, kLogRHi = 3.0;

__global__ void shadow_table_kernel(float* tab) {
    __shared__ float red[128];
    const int id = blockIdx.x;
    const int ia = id / (kTabT * kTabR), it = (id / kTabR) % kTabT, ir = id % kTabR;
    const double a = kAMax * ia / (kTabA - 1);
    const double th = kThLo + (kThHi - kThLo) * it / (kTabT - 1);
    const double r = pow(10.0, kLogRLo + (kLogRHi - kLogRLo) * ir / (kTabR - 1));
    float best = 0.0f;
    for (int k = threadIdx.x; k < kTabSamples; k += blockDim.x) {
        double al, be;
        if (critical_point(a, r, th, static_cast<double>(k) / (kTabSamples - 1), &al, &be))
            best = fmaxf(best, static_cast<float>(sqrt(al * al + be * be)));
    }
    red[threadIdx.x] = best;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) tab[id] = red[0];
}

__device__ __forceinline__ double uniform01(uint64_t seed, uint64_t k) {
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (k + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return static_cast<double>(z >> 11) * (1.0 / 9007199254740992.0);
}

__device__ __forceinline__ float table_lookup(const float* tab, double a, double th, double lr) {
    const double fa = fmin(fmax(a / kAMax, 0.0), 1.0) * (kTabA - 1);
    const double ft = fmin(fmax((th - kThLo) / (kThHi - kThLo), 0.0), 1.0) * (kTabT - 1);
    const double fr = fmin(fmax((lr - kLogRLo) / (kLogRHi - kLogRLo), 0.0), 1.0) * (kTabR - 1);
    const int i0 = min(static_cast<int>(fa), kTabA - 2), j0 = min(static_cast<int>(ft), kTabT - 2),
              k0 = min(static_cast<int>(fr), kTabR - 2);
    const double wa = fa - i0, wt = ft - j0, wr = fr - k0;
    double v = 0.0;
    for (int di = 0; di < 2; ++di)
        for (int dj = 0; dj < 2; ++dj)
            for (int dk = 0; dk < 2; ++dk) {
                const double w = (di ? wa : 1.0 - wa) * (dj ? wt : 1.0 - wt) * (dk ? wr : 1.0 - wr);
                v += w * tab[((i0 + di) * kTabT + (j0 + dj)) * kTabR + (k0 + dk)];
            }
    return static_cast<float>(v);
}

__global__ void sample_kernel(const float* __restrict__ tab, uint64_t seed, long long n, double* a, double* r,
                              double* th, double* al, double* be, float* x) {
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const uint64_t k = 6ull * static_cast<uint64_t>(i);
        const double ai = kAMax * uniform01(seed, k);
        const double ti = kThLo + (kThHi - kThLo) * uniform01(seed, k + 1);
        const double lr = kLogRLo + (kLogRHi - kLogRLo) * uniform01(seed, k + 2);
        const double ri = pow(10.0, lr);
        const double R = 1.5 * table_lookup(tab, ai, ti, lr);
        const double rad = R * sqrt(uniform01(seed, k + 3)), ang = 2.0 * kPi * uniform01(seed, k + 4);
        double sn, cs;
        sincos(ang, &sn, &cs);
        a[i] = ai;
        r[i] = ri;
        th[i] = ti;
        al[i] = rad * cs;
        be[i] = rad * sn;
        float* xi = x + 5 * i;
        xi[0] = static_cast<float>(ai);
        xi[1] = static_cast<float>(ti);
        xi[2] = static_cast<float>(log10(ri));
        xi[3] = static_cast<float>(rad * cs);
        xi[4] = static_cast<float>(rad * sn);
    }
}

// Classes and targets from tracer outputs (the convention of bhk_surrogate_train).
__global__ void label_kernel(long long n, const uint8_t* __restrict__ oc, const double* __restrict__ rd,
                             const double* __restrict__ g, const double* __restrict__ ti,
                             const double* __restrict__ pi, uint8_t* cls, float* tgt) {
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const uint8_t c = oc[i];
        float t[kOut] = {0, 0, 0, 0, 0, 0, 0, 0};
        if (c == BHK_RAY_DISK) {
            t[3] = static_cast<float>(rd[i] / 30.0);
            t[4] = static_cast<float>(log(fmax(g[i], 1e-30)));
        } else if (c == BHK_RAY_ESCAPED) {
            double s, co, sp, cp;
            sincos(ti[i], &s, &co);
            sincos(pi[i], &sp, &cp);
            t[5] = static_cast<float>(s * cp);
            t[6] = static_cast<float>(s * sp);
            t[7] = static_cast<float>(co);
        }
        cls[i] = c;
        for (int k = 0; k < kOut; ++k) tgt[kOut * i + k] = t[k];
    }
}

}  // namespace sur
}  // namespace bhk

extern "C" bhk_status bhk_surrogate_dataset(bhk_context* ctx, int64_t n, uint64_t seed, double r_disk_out,
                                            const bhk_trace_opts* opts, float* x, uint8_t* cls, float* target,
                                            double* rays5, void* stream) {
    using namespace bhk::sur;
    if (!ctx || n <= 0 || n > (int64_t(1) << 31) - 1 || !x || !cls || !target || !(r_disk_out >= 0.0)) {
        set_last_error("bhk_surrogate_dataset: bad arguments");
        return BHK_EINVAL;
    }
    cudaSetDevice(bhk::context_device(ctx));
    cudaStream_t st = bhk::context_stream(ctx, stream);  // the tracer below runs on the same stream
    float* tab = nullptr;
    double* d = rays5;
    uint8_t* oc = nullptr;
    double* o5 = nullptr;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&tab), sizeof(float) * kTabA * kTabT * kTabR);
    if (e == cudaSuccess && !rays5) e = cudaMalloc(reinterpret_cast<void**>(&d), sizeof(double) * 5 * n);
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&oc), n);
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&o5), sizeof(double) * 5 * n);
    bhk_status rs = BHK_OK;
    if (e == cudaSuccess) {
        shadow_table_kernel<<<kTabA * kTabT * kTabR, 128, 0, st>>>(tab);
        sample_kernel<<<1024, 256, 0, st>>>(tab, seed, n, d, d + n, d + 2 * n, d + 3 * n, d + 4 * n, x);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        bhk_trace_opts o{};
        if (opts) o = *opts;
        else o.precision = BHK_PREC_MIXED;
        bhk_rays_out out{};
        out.outcome = oc;
        out.r_disk = o5;
        out.phi_disk = o5 + n;
        out.g = o5 + 2 * n;
        out.theta_inf = o5 + 3 * n;
        out.phi_inf = o5 + 4 * n;
        rs = bhk_trace_rays(ctx, n, d, d + n, d + 2 * n, d + 3 * n, d + 4 * n, 0.0, r_disk_out, &o, &out, st);
        if (rs == BHK_OK) {
            label_kernel<<<1024, 256, 0, st>>>(n, oc, o5, o5 + 2 * n, o5 + 3 * n, o5 + 4 * n, cls, target);
            e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        }
    }
    if (tab) cudaFree(tab);
    if (d && d != rays5) cudaFree(d);
    if (oc) cudaFree(oc);
    if (o5) cudaFree(o5);
    if (rs != BHK_OK) return rs;
    if (e != cudaSuccess) {
        set_last_error(std::string("bhk_surrogate_dataset: ") + cudaGetErrorString(e));
        return BHK_ECUDA;
    }
    return BHK_OK;
}
