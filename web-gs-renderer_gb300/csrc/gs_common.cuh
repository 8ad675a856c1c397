// gs_common.cuh -- device helpers shared by the splat kernels of libwebgs.so.
//
// Every kernel is built with -fmad=false: a*b+c rounds twice unless written as __fmaf_rn, which
// keeps the fp32 results bit-identical to the pinned arithmetic of the reference restatement
// (WGSL source order, no contraction, the exp below).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gs {

// Device status word bits (also in gs.h as GS_DEV_*).
constexpr uint32_t kDevOverflow = 1u;
constexpr uint32_t kDevTimeout = 2u;
constexpr uint32_t kDevBounds = 4u;  // checked builds: a store index outside its buffer (the store is skipped)
constexpr uint32_t kDevCanary = 8u;  // checked builds: a canary pad around a device buffer was overwritten

// Checked builds (-DGS_CHECKED, libwebgs_checked.so) test every data-dependent store index against
// its buffer's size, skip the store and record kDevBounds instead of writing out of bounds; product
// builds compile the test away (their indices are bounded by construction).
#ifdef GS_CHECKED
#define GS_IN_BOUNDS(i, n, status) ((i) < (n) ? true : (atomicOr((status), ::gs::kDevBounds), false))
#else
#define GS_IN_BOUNDS(i, n, status) true
#endif

// Bounded spin: a wait on another CTA's publication gives up after this many polls (about a
// second with the back-off below; a healthy predecessor publishes within microseconds), records
// kDevTimeout and returns, so no kernel can hang the GPU.
constexpr uint32_t kSpinLimit = 1u << 20;

// Scene attribute rows of the device (structure-of-arrays) layout, one row of `stride` floats each.
constexpr int kRowPos = 0;      // x, y, z
constexpr int kRowScale = 3;    // log-scale 0..2
constexpr int kRowQuat = 6;     // rot_0..rot_3 as stored: (w, x, y, z)
constexpr int kRowDc = 10;      // f_dc_0..2
constexpr int kRowOpacity = 13; // opacity logit
constexpr int kRowRest = 14;    // f_rest_0..44 (channel-major: index c + 15*channel)
constexpr int kRows = 59;

// Constants of preprocess.wgsl:32-54 and raseter.wgsl:19-21, as the f32 literals.
constexpr float kSmallValue = 0.0000001f;
constexpr float kZNearView = 0.2f;
constexpr float kFrustumExtended = 1.3f;
constexpr float kShC0 = 0.28209479177387814f;
constexpr float kShC1 = 0.4886025119029199f;
constexpr float kShC2_0 = 1.0925484305920792f;
constexpr float kShC2_1 = -1.0925484305920792f;
constexpr float kShC2_2 = 0.31539156525252005f;
constexpr float kShC2_3 = -1.0925484305920792f;
constexpr float kShC2_4 = 0.5462742152960396f;
constexpr float kShC3_0 = -0.5900435899266435f;
constexpr float kShC3_1 = 2.890611442640554f;
constexpr float kShC3_2 = -0.4570457994644658f;
constexpr float kShC3_3 = 0.3731763325901154f;
constexpr float kShC3_4 = -0.4570457994644658f;
constexpr float kShC3_5 = 1.445305721320277f;
constexpr float kShC3_6 = -0.5900435899266435f;
constexpr float kAlphaClamp = 0.99f;
constexpr float kEpsilon = 0x1.010102p-8f;  // 1.0f / 255.0f
constexpr float kBlendThreshold = 0.0001f;

// The 176-byte GlobalUniforms block (preprocess.wgsl:2-12).
struct ViewBlock {
    float view[16];
    float viewProj[16];
    float cameraPos[3];
    uint32_t count;
    float focal[2];
    float tanFov[2];
    float textureSize[2];
    uint32_t pad0, pad1;
};
static_assert(sizeof(ViewBlock) == 176, "GlobalUniforms is 176 bytes");

// Pinned fp32 exp: exp(x) = 2^n e^r, n = rint(x log2 e), r = x - n ln2 with ln2 split into two f32
// parts (one fma each), e^r by its Taylor series to degree 7 in Horner form (|r| <= ln2/2, so the
// truncation error stays below 6e-9 relative), 2^n applied as two exact power-of-two factors so a
// subnormal result rounds once. Every step is an IEEE-754 operation, so the value is the same on
// any conforming host or device.
__device__ __forceinline__ float pinned_expf(float x) {
    if (x != x) return x;
    if (x > 89.0f) return __int_as_float(0x7f800000);
    if (x < -104.0f) return 0.0f;
    const float n = rintf(__fmul_rn(x, 0x1.715476p+0f));
    float r = __fmaf_rn(-n, 0x1.62e43p-1f, x);
    r = __fmaf_rn(-n, -0x1.05c61p-29f, r);
    float p = 0x1.a01a02p-13f;
    p = __fmaf_rn(p, r, 0x1.6c16c2p-10f);
    p = __fmaf_rn(p, r, 0x1.111112p-7f);
    p = __fmaf_rn(p, r, 0x1.555556p-5f);
    p = __fmaf_rn(p, r, 0x1.555556p-3f);
    p = __fmaf_rn(p, r, 0.5f);
    p = __fmaf_rn(p, r, 1.0f);
    p = __fmaf_rn(p, r, 1.0f);
    const int k = (int)n;
    const int k1 = k / 2;
    const int k2 = k - k1;
    return __fmul_rn(__fmul_rn(p, __int_as_float((k1 + 127) << 23)), __int_as_float((k2 + 127) << 23));
}

// 64-bit relaxed device-scope load/store for lookback words (the value travels in the word).
__device__ __forceinline__ uint64_t ld_relaxed_u64(const uint64_t* p) {
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_u64(uint64_t* p, uint64_t v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Lookback word: [63:34] sequence number of the pass that wrote it, [33:32] flag, [31:0] value.
// Words of earlier passes carry an older sequence number and read as "not ready", so the flag
// arrays are zeroed at allocation and not per pass (sequence numbers start at 16); they are cleared
// again only on the frame where the 30-bit tags wrap to zero (k_frame_begin).
constexpr uint32_t kFlagAggregate = 1u;
constexpr uint32_t kFlagInclusive = 2u;
constexpr uint32_t kSeqMask = (1u << 30) - 1u;
__device__ __forceinline__ uint64_t make_word(uint32_t seq, uint32_t flag, uint32_t value) {
    return ((uint64_t)(seq & kSeqMask) << 34) | ((uint64_t)flag << 32) | (uint64_t)value;
}
__device__ __forceinline__ uint32_t word_seq(uint64_t w) { return (uint32_t)(w >> 34); }
__device__ __forceinline__ uint32_t word_flag(uint64_t w) { return (uint32_t)(w >> 32) & 3u; }
__device__ __forceinline__ uint32_t word_value(uint64_t w) { return (uint32_t)w; }

// Exclusive prefix of partition `part` over the words of its predecessors (decoupled lookback),
// executed by one full warp: lane i inspects predecessor part-1-i, the warp stops at the nearest
// inclusive word and sums the aggregates above it. Every wait is bounded; on timeout the status
// word gets kDevTimeout and the missing word counts as an inclusive zero.
__device__ __forceinline__ uint32_t warp_lookback(const uint64_t* words, uint32_t part, uint32_t seq,
                                                  uint32_t* status) {
    const int lane = threadIdx.x & 31;
    uint32_t excl = 0;
    int64_t top = (int64_t)part - 1;
    const uint32_t want = seq & kSeqMask;
    while (true) {
        const int64_t idx = top - lane;
        uint32_t flag = kFlagInclusive, value = 0;
        if (idx >= 0) {
            uint32_t spins = 0;
            uint64_t w = ld_relaxed_u64(words + idx);
            while (word_seq(w) != want || word_flag(w) == 0u) {
                if (++spins > kSpinLimit) {
                    atomicOr(status, kDevTimeout);
                    w = make_word(want, kFlagInclusive, 0u);
                    break;
                }
                if (spins > 64u) __nanosleep(64);
                w = ld_relaxed_u64(words + idx);
            }
            flag = word_flag(w);
            value = word_value(w);
        }
        const uint32_t inc = __ballot_sync(0xffffffffu, flag == kFlagInclusive);
        uint32_t contrib = value;
        if (inc) {
            const int first = __ffs(inc) - 1;
            if (lane > first) contrib = 0;
        }
        for (int o = 16; o > 0; o >>= 1) contrib += __shfl_xor_sync(0xffffffffu, contrib, o);
        excl += contrib;
        if (inc) break;
        top -= 32;
    }
    return excl;
}

// ---- bulk-copy (TMA) staging helpers ------------------------------------------------------------
// Programmatic dependent launch (griddepcontrol): a kernel launched with launch_pdl calls pdl_wait()
// before touching anything; it returns once the kernel before it on the stream has completed and its
// writes are visible (at once for a kernel launched without the attribute). No kernel triggers its
// dependents early: an explicit trigger at the top of every kernel measured slower in the frame's graph
// (its dependents' CTAs sat in the wait), while the implicit trigger as CTAs exit keeps the gain.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// global -> shared bulk copy completing on `bar`; addresses 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
    uint32_t ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(ok) : "r"(smem_u32(bar)), "r"(phase) : "memory");
    return ok != 0;
}

// Frame control block in device memory, reset by k_frame_begin at the start of every frame.
struct FrameCtl {
    uint32_t seq;            // sequence number of the current pass group (incremented per frame)
    uint32_t status;         // kDev* bits
    uint32_t instance_count; // I (unclamped)
    uint32_t sorted_count;   // min(I, max_instance)
    uint32_t visible;        // Gaussians with tilesTouched > 0
    uint32_t near_pass;      // Gaussians in front of the near plane (their full record is read)
    uint32_t tickets[15];    // partition tickets, one per ticketed kernel launch of the frame
    uint32_t hist[8 * 256];  // per-pass digit histograms of the sort (passes x radix)
};

}  // namespace gs
