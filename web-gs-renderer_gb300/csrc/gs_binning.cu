// gs_binning.cu -- offset scan, emit, radix sort and tile ranges of the splat pipeline:
//   offset scan  src/shaders/offset_scan.wgsl:22-67   -> k_scan_emit (single pass: each partition sums
//                                                        its predecessors' published aggregates)
//   emit         src/shaders/emit.wgsl:28-66          -> k_scan_emit (fused, load-balanced)
//   indirect arg src/shaders/indirect_arg.wgsl:14-27  -> FrameCtl counts read on the device
//   radix sort   src/shaders/radix_parallel.wgsl      -> k_onesweep (one kernel per digit pass,
//                                                        per-digit prefixes from an aggregate tree)
//   tile ranges  src/shaders/tile_ranges.wgsl:7-34    -> the last k_onesweep pass (run bounds by
//                                                        min / max) + k_tile_place (empty tiles)
//   range clear  renderer.js:919                      -> k_frame_begin(_multi) (with the counters reset)
//
// Ordering: every kernel that chains partitions takes a ticket from FrameCtl so that partition p
// only ever waits on partitions already owned by running CTAs; every wait is bounded (kSpinLimit
// polls, then the timeout status is set and the wait ends).
#include <algorithm>
#include <atomic>

#include "gs_kernels.h"

namespace gs {
namespace {

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

// Block-wide exclusive scan of one value per thread (THREADS a multiple of 32). Returns the
// exclusive prefix; *total receives the block sum. Uses `warp_sums` (THREADS/32 words).
// Exclusive max-scan over the block (identity 0); warp_sums holds THREADS / 32 + 1 words.
template <int THREADS>
__device__ __forceinline__ uint32_t block_exclusive_max(uint32_t v, uint32_t* warp_sums) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl = max(incl, t);
    }
    uint32_t excl = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane == 0) excl = 0u;
    __syncthreads();
    if (lane == 31u) warp_sums[warp] = incl;
    __syncthreads();
    uint32_t prior = 0u;
    for (uint32_t w = 0; w < warp; ++w) prior = max(prior, warp_sums[w]);
    __syncthreads();
    return max(prior, excl);
}

template <int THREADS>
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* warp_sums, uint32_t* total) {
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += t;
    }
    if (lane == 31u) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        constexpr int kWarps = THREADS / 32;
        uint32_t s = lane < (uint32_t)kWarps ? warp_sums[lane] : 0u;
        uint32_t si = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, si, o);
            if (lane >= (uint32_t)o) si += t;
        }
        if (lane < (uint32_t)kWarps) warp_sums[lane] = si - s;  // exclusive warp offsets
        if (lane == (uint32_t)kWarps - 1u) warp_sums[kWarps] = si;
    }
    __syncthreads();
    const uint32_t r = warp_sums[warp] + incl - v;
    *total = warp_sums[THREADS / 32];
    __syncthreads();
    return r;
}

// Resets one frame's control block (CTA 0) and clears its tile ranges (renderer.js:919) with
// 16-byte stores across the CTAs [0, ncta), the tail word by word. A range is cleared to
// (0xFFFFFFFF, 0), the identities of the min / max the last sort pass combines the tile's bounds with;
// the tile order kernel writes (0, 0), the reference's cleared value, back into the tiles left empty.
//
// Lookback words carry only the low 30 bits of the sequence number, which advances by 16 per frame,
// so the tags repeat every 2^26 frames: a word left from 2^26 frames earlier with a set flag would
// read as published by the current frame. On the frame whose tags start again at zero, CTA 0 clears
// the frame's lookback words (`flags`, flag_words words) before any later kernel of the frame can
// read them. That is one clear every 2^26 frames, on the device, so replayed graphs are covered too.
__device__ __forceinline__ void frame_begin(FrameCtl* ctl, uint32_t* ranges, uint32_t range_words, uint64_t* flags,
                                            uint32_t flag_words, uint32_t cta, uint32_t ncta) {
    const uint32_t t = threadIdx.x;
    const uint32_t quads = range_words / 4u;  // range_words is even: (start, end) pairs
    for (uint32_t q = cta * blockDim.x + t; q < quads; q += ncta * blockDim.x)
        reinterpret_cast<uint4*>(ranges)[q] = make_uint4(0xFFFFFFFFu, 0u, 0xFFFFFFFFu, 0u);
    if (cta != 0) return;
    for (uint32_t i = quads * 4u + t; i < range_words; i += blockDim.x) ranges[i] = (i & 1u) ? 0u : 0xFFFFFFFFu;
    const uint32_t next = (ctl->seq & ~15u) + 16u;
    __syncthreads();  // every thread has read the old sequence number before thread 0 replaces it
    if (t == 0) {
        ctl->seq = next;
        ctl->status = 0u;
        ctl->instance_count = 0u;
        ctl->sorted_count = 0u;
        ctl->visible = 0u;
        ctl->near_pass = 0u;
    }
    if (t < 15) ctl->tickets[t] = 0u;
    for (uint32_t i = t; i < 8u * 256u; i += blockDim.x) ctl->hist[i] = 0u;
    if ((next & kSeqMask) == 0u && flags)
        for (uint32_t i = t; i < flag_words; i += blockDim.x) flags[i] = 0ull;
}

__global__ void k_frame_begin(FrameCtl* ctl, uint32_t* ranges, uint32_t range_words, uint64_t* flags,
                              uint32_t flag_words) {
    pdl_wait();
    frame_begin(ctl, ranges, range_words, flags, flag_words, blockIdx.x, gridDim.x);
}

__global__ void k_frame_begin_multi(MultiViewFrames mv) {
    pdl_wait();
    const uint32_t v = blockIdx.y;
    frame_begin(mv.ctl[v], mv.ranges[v], mv.range_words[v], mv.flags[v], mv.flag_words[v], blockIdx.x, gridDim.x);
}

// ---- fused offset scan + emit ---------------------------------------------------------------
// Partition p covers entries [p*2048, p*2048+2048) of counts[0..n] (n+1 entries; counts[n] = 0).
// 1. each thread loads 8 consecutive counts (two 16-byte loads), the block scans them;
// 2. the partition publishes its aggregate and sums its predecessors' aggregates in parallel;
// 3. offsets[g] are written (offsets[n] = I), the partition holding entry n publishes I and
//    min(I, max_instance) to FrameCtl (indirect_arg.wgsl:14-27);
// 4. the partition's instances [excl, excl + total) are emitted by all 256 threads in slot order,
//    each slot finding its Gaussian in an owner map built per chunk of slots, so one large splat
//    never serialises a warp; keys are ((ty*tilesPerRow + tx) << 16) | depth16 in row-major tile
//    order (emit.wgsl:55-66) and slots >= max_instance are dropped (:57-59);
// 5. the digit histograms of every sort pass are accumulated on the fly (per Gaussian for the
//    depth digits, per instance for the tile digits).
__global__ void __launch_bounds__(kScanThreads) k_scan_emit(const uint32_t* __restrict__ counts,
                                                            const uint4* __restrict__ meta, uint32_t n,
                                                            uint32_t tiles_x, uint32_t max_instance,
                                                            uint32_t digit_bits, uint32_t passes,
                                                            uint32_t* __restrict__ offsets, uint32_t* __restrict__ keys,
                                                            uint32_t* __restrict__ vals, FrameCtl* ctl,
                                                            uint64_t* flags, uint32_t slot) {
    __shared__ uint32_t s_off[kScanPartition + 1];
    __shared__ uint2 s_meta[kScanPartition];  // (minX | minY << 16, rect width | depth16 << 16)
    __shared__ uint32_t s_own[kScanPartition];  // owner (local Gaussian) of each slot of an emit chunk
    __shared__ uint32_t s_hist[8 * 256];
    __shared__ uint32_t s_warp[kScanThreads / 32 + 1];
    __shared__ uint32_t s_part, s_excl, s_seq;

    // the ticket counter and the sequence number were set by the frame's first kernel, two launches
    // back: the partition is taken before the wait for the preprocess, whose counts are read after it
    const uint32_t tid = threadIdx.x;
    if (tid == 0) {
        s_part = atomicAdd(&ctl->tickets[slot], 1u);
        s_seq = ctl->seq + slot;
    }
    const uint32_t radix = 1u << digit_bits;
    for (uint32_t i = tid; i < passes * radix; i += kScanThreads) s_hist[i] = 0u;
    pdl_wait();
    __syncthreads();
    const uint32_t part = s_part, seq = s_seq;
    const uint32_t entries = n + 1u;
    const uint32_t base = part * kScanPartition;
    const uint32_t g0 = base + tid * kScanItems;

    uint32_t c[kScanItems];
    if (g0 + kScanItems <= entries) {
        const uint4 a = *reinterpret_cast<const uint4*>(counts + g0);
        const uint4 b = *reinterpret_cast<const uint4*>(counts + g0 + 4);
        c[0] = a.x; c[1] = a.y; c[2] = a.z; c[3] = a.w; c[4] = b.x; c[5] = b.y; c[6] = b.z; c[7] = b.w;
    } else {
#pragma unroll
        for (uint32_t k = 0; k < kScanItems; ++k) c[k] = (g0 + k < entries) ? counts[g0 + k] : 0u;
    }
    uint32_t tsum = 0, vis = 0;
#pragma unroll
    for (uint32_t k = 0; k < kScanItems; ++k) {
        tsum += c[k];
        vis += c[k] != 0u ? 1u : 0u;
    }
    uint32_t total;
    const uint32_t texcl = block_exclusive_scan<kScanThreads>(tsum, s_warp, &total);

    // publish the aggregate at once; the local offsets and rects are staged while predecessors do
    // the same
    if (tid == 0) st_relaxed_u64(flags + part, make_word(seq, kFlagAggregate, total));
    // local offsets and rects into shared memory
    {
        uint32_t run = texcl;
#pragma unroll
        for (uint32_t k = 0; k < kScanItems; ++k) {
            const uint32_t lg = tid * kScanItems + k;
            s_off[lg] = run;
            if (c[k] != 0u) {
                const uint4 m = meta[g0 + k];
                const uint32_t width = (m.y & 0xFFFFu) - (m.x & 0xFFFFu) + 1u;
                s_meta[lg] = make_uint2(m.x, width | (m.z << 16u));
            }
            run += c[k];
        }
        if (tid == 0) s_off[kScanPartition] = total;
    }
    // sum the aggregates of all predecessors: every partition publishes before it waits on anything
    // and its predecessors hold smaller tickets (they are running or done), so the waits end without
    // a chain of inclusive prefixes; one word per thread per 256 predecessors is read
    {
        const uint32_t want = seq & kSeqMask;
        uint32_t psum = 0;
        for (uint32_t j = tid; j < part; j += kScanThreads) {
            const uint64_t* p = flags + j;
            uint64_t w = ld_relaxed_u64(p);
            uint32_t spins = 0;
            while (word_seq(w) != want || word_flag(w) == 0u) {
                if (++spins > kSpinLimit) {  // bounded: record the timeout and count the partition as empty
                    atomicOr(&ctl->status, kDevTimeout);
                    w = make_word(want, kFlagAggregate, 0u);
                    break;
                }
                if (spins > 64u) __nanosleep(64);
                w = ld_relaxed_u64(p);
            }
            psum += word_value(w);
        }
        uint32_t excl_sum;
        block_exclusive_scan<kScanThreads>(psum, s_warp, &excl_sum);
        if (tid == 0) s_excl = excl_sum;
    }
    if (vis) atomicAdd(&ctl->visible, vis);
    __syncthreads();
    const uint32_t excl = s_excl;

    // offsets (the debug view of offset_scan.wgsl's in-place result)
#pragma unroll
    for (uint32_t k = 0; k < kScanItems; ++k) {
        const uint32_t g = g0 + k;
        if (g < entries) offsets[g] = excl + s_off[tid * kScanItems + k];
        if (g == n) {
            const uint32_t I = excl + s_off[tid * kScanItems + k];
            ctl->instance_count = I;
            ctl->sorted_count = I < max_instance ? I : max_instance;
            if (I > max_instance) atomicOr(&ctl->status, kDevOverflow);
        }
    }

    // digits of the depth bits depend on the Gaussian only: one histogram add per Gaussian, weighted
    // by its kept instances (slots below max_instance); the tile digits are counted per instance
    const uint32_t mask = radix - 1u;
    const uint32_t depth_passes = min(passes, 16u / digit_bits);
#pragma unroll
    for (uint32_t k = 0; k < kScanItems; ++k) {
        const uint32_t lg = tid * kScanItems + k;
        if (c[k] == 0u) continue;
        const uint32_t first = excl + s_off[lg];
        const uint32_t kept = first >= max_instance ? 0u : min(c[k], max_instance - first);
        if (kept == 0u) continue;
        const uint32_t d16 = s_meta[lg].y >> 16u;
        for (uint32_t p = 0; p < depth_passes; ++p)
            atomicAdd(&s_hist[p * radix + ((d16 >> (p * digit_bits)) & mask)], kept);
    }

    // emit, in chunks of kScanPartition slots: the owner of every slot of a chunk comes from an owner
    // map (each Gaussian marks the slot where its run starts, or slot 0 if its run covers the chunk's
    // start; an inclusive max-scan fills the rest, local indices growing with their offsets), so no
    // slot searches; the tile of instance k of a w-wide rect is (k / w, k % w) through a float
    // reciprocal corrected to the exact quotient
    const uint32_t kept_total = excl >= max_instance ? 0u : min(total, max_instance - excl);
    for (uint32_t c0 = 0; c0 < kept_total; c0 += kScanPartition) {
        const uint32_t c1 = c0 + kScanPartition;
#pragma unroll
        for (uint32_t k = 0; k < kScanItems; ++k) s_own[tid * kScanItems + k] = 0u;
        __syncthreads();
#pragma unroll
        for (uint32_t k = 0; k < kScanItems; ++k) {
            const uint32_t lg = tid * kScanItems + k;
            if (c[k] == 0u) continue;
            const uint32_t start = s_off[lg];
            if (start >= c0 && start < c1) s_own[start - c0] = lg;
            else if (start < c0 && start + c[k] > c0) s_own[0] = lg;
        }
        __syncthreads();
        uint32_t run = 0;
#pragma unroll
        for (uint32_t k = 0; k < kScanItems; ++k) run = max(run, s_own[tid * kScanItems + k]);
        const uint32_t before = block_exclusive_max<kScanThreads>(run, s_warp);
        run = before;
#pragma unroll
        for (uint32_t k = 0; k < kScanItems; ++k) {
            run = max(run, s_own[tid * kScanItems + k]);
            s_own[tid * kScanItems + k] = run;
        }
        __syncthreads();
        const uint32_t cn = min(kept_total - c0, kScanPartition);
        for (uint32_t j = tid; j < cn; j += kScanThreads) {
            const uint32_t i = c0 + j;
            const uint32_t lg = s_own[j];
            const uint32_t k = i - s_off[lg];
            const uint2 m = s_meta[lg];
            const uint32_t w = m.y & 0xFFFFu;
            // k < 2^24 and w < 2^16 are exact floats; the rounded quotient is off by at most one
            uint32_t q = (uint32_t)__fdividef((float)k, (float)w);
            int32_t r = (int32_t)(k - q * w);
            if (r < 0) { --q; r += (int32_t)w; }
            else if (r >= (int32_t)w) { ++q; r -= (int32_t)w; }
            const uint32_t ty = (m.x >> 16u) + q, tx = (m.x & 0xFFFFu) + (uint32_t)r;
            const uint32_t key = ((ty * tiles_x + tx) << 16u) | (m.y >> 16u);
            if (GS_IN_BOUNDS(excl + i, max_instance, &ctl->status)) {
                keys[excl + i] = key;
                vals[excl + i] = base + lg;
            }
            for (uint32_t p = depth_passes; p < passes; ++p)
                atomicAdd(&s_hist[p * radix + ((key >> (p * digit_bits)) & mask)], 1u);
        }
        __syncthreads();
    }
    __syncthreads();
    for (uint32_t i = tid; i < passes * radix; i += kScanThreads)
        if (s_hist[i]) atomicAdd(&ctl->hist[i], s_hist[i]);
}

// ---- standalone exclusive scan (offset_scan.wgsl:22-67 semantics, any n) ------------------------
__global__ void __launch_bounds__(kScanThreads) k_exclusive_scan(uint32_t* data, uint32_t n, uint32_t* total_out,
                                                                 FrameCtl* ctl, uint64_t* flags, uint32_t slot) {
    __shared__ uint32_t s_warp[kScanThreads / 32 + 1];
    __shared__ uint32_t s_part, s_excl, s_seq;
    const uint32_t tid = threadIdx.x;
    if (tid == 0) {
        s_part = atomicAdd(&ctl->tickets[slot], 1u);
        s_seq = ctl->seq + slot;
    }
    __syncthreads();
    const uint32_t part = s_part, seq = s_seq;
    const uint32_t g0 = part * kScanPartition + tid * kScanItems;
    uint32_t c[kScanItems], tsum = 0;
#pragma unroll
    for (uint32_t k = 0; k < kScanItems; ++k) {
        c[k] = (g0 + k < n) ? data[g0 + k] : 0u;
        tsum += c[k];
    }
    uint32_t total;
    const uint32_t texcl = block_exclusive_scan<kScanThreads>(tsum, s_warp, &total);
    if (tid < 32) {
        if (tid == 0) st_relaxed_u64(flags + part, make_word(seq, part == 0 ? kFlagInclusive : kFlagAggregate, total));
        const uint32_t excl = warp_lookback(flags, part, seq, &ctl->status);
        if (tid == 0) {
            if (part != 0) st_relaxed_u64(flags + part, make_word(seq, kFlagInclusive, excl + total));
            s_excl = excl;
        }
    }
    __syncthreads();
    uint32_t run = s_excl + texcl;
#pragma unroll
    for (uint32_t k = 0; k < kScanItems; ++k) {
        if (g0 + k < n) data[g0 + k] = run;
        run += c[k];
    }
    if (part == gridDim.x - 1u && tid == kScanThreads - 1u) *total_out = run;
}

// ---- digit histograms for a standalone sort ---------------------------------------------------
// Only the low key_bits bits take part: the last pass's digit is masked to the bits left.
__global__ void k_digit_hist(const uint32_t* __restrict__ keys, uint32_t n, uint32_t digit_bits, uint32_t key_bits,
                             uint32_t* hist) {
    __shared__ uint32_t s_hist[8 * 256];
    const uint32_t radix = 1u << digit_bits;
    const uint32_t passes = (key_bits + digit_bits - 1u) / digit_bits;
    for (uint32_t i = threadIdx.x; i < passes * radix; i += blockDim.x) s_hist[i] = 0u;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t key = keys[i];
        for (uint32_t p = 0; p < passes; ++p) {
            const uint32_t left = key_bits - p * digit_bits;
            const uint32_t mask = left >= digit_bits ? radix - 1u : (1u << left) - 1u;
            atomicAdd(&s_hist[p * radix + ((key >> (p * digit_bits)) & mask)], 1u);
        }
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < passes * radix; i += blockDim.x)
        if (s_hist[i]) atomicAdd(&hist[i], s_hist[i]);
}

// Sum of the values of `count` (1..7) tagged words p[0], p[-stride], ..., p[-(count-1) stride]: every
// load is issued before the first is checked, and the words still without this pass's tag are polled
// together (one memory round trip per poll for all of them), so the sum is ready one round trip after
// the last of them is published. Bounded: on expiry the timeout is recorded and the words still
// missing count as zero.
__device__ __forceinline__ uint32_t sum_tagged(const uint64_t* p, size_t stride, uint32_t count, uint32_t want,
                                               uint32_t* status) {
    uint64_t w[7];
#pragma unroll
    for (uint32_t q = 0; q < 7u; ++q) w[q] = q < count ? ld_relaxed_u64(p - q * stride) : 0ull;
    auto ready = [&](uint64_t v) { return word_seq(v) == want && word_flag(v) != 0u; };
    uint32_t spins = 0;
    while (true) {
        bool all = true;
#pragma unroll
        for (uint32_t q = 0; q < 7u; ++q) all = all && (q >= count || ready(w[q]));
        if (all) break;
        if (++spins > kSpinLimit) {
            atomicOr(status, kDevTimeout);
            break;
        }
        if (spins > 64u) __nanosleep(64);
#pragma unroll
        for (uint32_t q = 0; q < 7u; ++q)
            if (q < count && !ready(w[q])) w[q] = ld_relaxed_u64(p - q * stride);
    }
    uint32_t sum = 0;
#pragma unroll
    for (uint32_t q = 0; q < 7u; ++q)
        if (q < count && ready(w[q])) sum += word_value(w[q]);
    return sum;
}

// ---- onesweep radix pass ------------------------------------------------------------------------
// One stable counting-sort pass on digit (key >> shift) & (RADIX-1) (radix_parallel.wgsl:26-160 in
// one kernel). Persistent CTAs take partitions of 256 x ITEMS keys (4096 or 2048) by ticket. Per
// partition:
//   - keys load warp-striped (item k of lane l of warp w is element w*32*ITEMS + k*32 + l), so every
//     load is a 128-byte line and the warp processes its elements in index order;
//   - __match_any_sync groups the lanes holding the same digit; a lane's rank is the count of
//     equal digits in earlier items of its warp plus its rank among the equal lanes (stable). The
//     match costs more the more distinct values the warp holds: with SPLIT > 0 it matches only the
//     digit's high bits and separates the low SPLIT bits with one ballot each (measured on the
//     1M / 1080p frame: the tile digits of keys in depth order are nearly all distinct within a
//     warp, and their two passes take 16 us less per frame with SPLIT = w/2 of a w-bit digit, while
//     the depth passes, whose warps hold few distinct digits, are fastest with the plain match);
//   - ranks (< 4096) are kept two per register, which keeps the thread within 64 registers;
//   - per-digit warp counts are scanned across warps (warp order = index order) and the CTA's digit
//     totals are published; every digit's count in the earlier partitions comes from a tree of
//     aggregates built inside the pass (one thread per digit): level 0 holds the partitions' totals,
//     level L+1 the sums of groups of 8 level-L nodes, each published by the partition that completes
//     the group; partition p sums the earlier siblings of its node at every level (the base-8 digits
//     of p: at most 7 words per level, loaded together). All partitions of a pass publish their
//     totals at about the same time, so the prefixes are ready a few memory round trips later at
//     every partition, where a decoupled lookback passes inclusive prefixes along the partitions a
//     few per round trip (on the 1M / 1080p frame the last of 536 partitions waited about 7 us);
//   - keys/values are staged in shared memory in local sorted order and written out at
//     global_digit_base + rank, which keeps runs of equal digits contiguous in global memory.
template <int BITS, int ITEMS, int SPLIT>
__global__ void __launch_bounds__(kSortThreads, 4) k_onesweep(const uint32_t* __restrict__ keys_in,
                                                           const uint32_t* __restrict__ vals_in,
                                                           uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out,
                                                           const uint32_t* n_dev, uint32_t n_host, uint32_t shift,
                                                           uint32_t dmask, const uint32_t* __restrict__ hist,
                                                           FrameCtl* ctl, uint64_t* flags, uint32_t slot,
                                                           uint32_t early, uint32_t* __restrict__ ranges,
                                                           uint32_t tiles) {
    // early: n, the histogram and the ticket counter were written before the previous kernel, so
    // each CTA takes its first partition and computes the digit bases before waiting for that
    // kernel (only the keys and values it wrote are read after the wait)
    if (!early) pdl_wait();
    constexpr uint32_t RADIX = 1u << BITS;
    const uint32_t MASK = dmask & (RADIX - 1u);  // digit mask of this pass (narrower on a last partial digit)
    constexpr uint32_t WARPS = kSortThreads / 32;
    constexpr uint32_t PER_WARP = ITEMS * 32;
    constexpr uint32_t PART = kSortThreads * ITEMS;  // keys per partition
    __shared__ uint32_t s_keys[PART];
    __shared__ uint32_t s_vals[PART];
    __shared__ uint32_t s_whist[WARPS][RADIX];
    __shared__ uint32_t s_gbase[RADIX];     // global exclusive digit base of this pass
    __shared__ uint32_t s_out[RADIX];       // global position of local element 0 of each digit
    __shared__ uint32_t s_warp[WARPS + 1];
    __shared__ uint32_t s_part, s_seq;

    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t n = n_dev ? *n_dev : n_host;
    const uint32_t nparts = (n + PART - 1u) / PART;
    // the grid is sized before n is known: CTAs past the partition count leave without taking a
    // ticket (CTAs 0..nparts-1 take every partition between them, in ticket order), so they add no
    // traffic on the ticket counter the working CTAs draw from
    if (blockIdx.x >= nparts) return;

    if (tid == 0) s_seq = ctl->seq + slot;
    bool have_bases = false, waited = early == 0u;

    while (true) {
        __syncthreads();
        if (tid == 0) s_part = atomicAdd(&ctl->tickets[slot], 1u);
        __syncthreads();
        const uint32_t part = s_part, seq = s_seq;
        if (part >= nparts) break;  // CTAs left without a partition exit before any other work
        if (!have_bases) {
            // global digit bases of this pass: exclusive scan of the histogram
            const uint32_t h = tid < RADIX ? hist[tid] : 0u;
            uint32_t tot;
            const uint32_t ex = block_exclusive_scan<kSortThreads>(h, s_warp, &tot);
            if (tid < RADIX) s_gbase[tid] = ex;
            have_bases = true;
        }
        if (!waited) {
            pdl_wait();
            waited = true;
        }
        const uint32_t base = part * PART;
        const uint32_t valid_n = min(PART, n - base);

        for (uint32_t d = lane; d < RADIX; d += 32) s_whist[warp][d] = 0u;
        __syncwarp();

        uint32_t key[ITEMS];
        uint32_t rank2[ITEMS / 2];  // rank of item k in bits 16*(k&1) of rank2[k/2]
#pragma unroll
        for (uint32_t k = 0; k < ITEMS / 2; ++k) rank2[k] = 0u;
        const uint32_t wbase = base + warp * PER_WARP;
#pragma unroll
        for (uint32_t k = 0; k < ITEMS; ++k) {
            const uint32_t idx = wbase + k * 32u + lane;
            key[k] = idx < n ? keys_in[idx] : 0xFFFFFFFFu;
        }
#pragma unroll
        for (uint32_t k = 0; k < ITEMS; ++k) {
            const uint32_t idx = wbase + k * 32u + lane;
            const bool ok = idx < n;
            const uint32_t d = ok ? ((key[k] >> shift) & MASK) : RADIX;  // RADIX marks padding
            // the padding marker's high part (RADIX >> SPLIT) differs from every digit's
            uint32_t peers = __match_any_sync(0xffffffffu, d >> SPLIT);
#pragma unroll
            for (int b = 0; b < SPLIT; ++b) {
                const bool bit = (d >> b) & 1u;
                const uint32_t bal = __ballot_sync(0xffffffffu, bit);
                peers &= bit ? bal : ~bal;
            }
            const uint32_t pre = ok ? s_whist[warp][d] : 0u;
            __syncwarp();
            if (ok) {
                const uint32_t below = peers & ((1u << lane) - 1u);
                if (below == 0u) s_whist[warp][d] = pre + __popc(peers);
                rank2[k / 2] |= (pre + __popc(below)) << (16u * (k & 1u));
            }
            __syncwarp();
        }
        __syncthreads();

        // per digit: exclusive over warps, CTA total (published at once, level 0 of the tree)
        uint32_t cta_total = 0;
        if (tid < RADIX) {
#pragma unroll
            for (uint32_t w = 0; w < WARPS; ++w) {
                const uint32_t c = s_whist[w][tid];
                s_whist[w][tid] = cta_total;
                cta_total += c;
            }
            st_relaxed_u64(flags + (size_t)part * RADIX + tid, make_word(seq, kFlagAggregate, cta_total));
        }
        uint32_t dtot;
        const uint32_t dstart = block_exclusive_scan<kSortThreads>(tid < RADIX ? cta_total : 0u, s_warp, &dtot);
        if (tid < RADIX) {
            // each warp's slot base of this digit: the digit's local sorted start plus the warps before
#pragma unroll
            for (uint32_t w = 0; w < WARPS; ++w) s_whist[w][tid] += dstart;
        }
        // the digit's count in all earlier partitions, from the aggregate tree (one thread per digit,
        // bounded waits): at level L the earlier siblings of the partition's own node are summed (the
        // base-8 digit L of its index, at most 7 words, loaded together), and the partition whose node
        // completes a group of 8 publishes the group's sum one level up
        auto prefix = [&]() {
            const uint32_t want = seq & kSeqMask;
            uint32_t excl = 0, node = cta_total, idx = part, rows = nparts;
            size_t base = 0;
            bool completes = true;  // this partition is the last one of its node at the current level
            while (idx) {
                const uint32_t a = idx & 7u;
                const uint32_t sib =
                    a ? sum_tagged(flags + base + (size_t)(idx - 1u) * RADIX + tid, RADIX, a, want, &ctl->status) : 0u;
                excl += sib;
                completes = completes && a == 7u;
                base += (size_t)rows * RADIX;
                rows = (rows + 7u) >> 3;
                idx >>= 3;
                if (completes) {
                    node += sib;
                    st_relaxed_u64(flags + base + (size_t)idx * RADIX + tid, make_word(seq, kFlagAggregate, node));
                }
            }
            s_out[tid] = s_gbase[tid] + excl - dstart;
        };
        // a partition that completes a group of 8 builds its tree nodes at once; the others first put
        // their keys in local sorted order, which needs no global prefix, and read the tree after
        // that, when more of it is complete
        const bool builds = (part & 7u) == 7u;
        if (builds && tid < RADIX) prefix();
        __syncthreads();

        // local sorted order in shared memory; values are read only now, straight into their slot,
        // which keeps them out of registers during the ranking
#pragma unroll
        for (uint32_t k = 0; k < ITEMS; ++k) {
            const uint32_t idx = wbase + k * 32u + lane;
            if (idx < n) {
                const uint32_t d = (key[k] >> shift) & MASK;
                const uint32_t pos = s_whist[warp][d] + ((rank2[k / 2] >> (16u * (k & 1u))) & 0xFFFFu);
                s_keys[pos] = key[k];
                s_vals[pos] = vals_in[idx];
            }
        }
        if (!builds && tid < RADIX) prefix();
        __syncthreads();
        for (uint32_t i = tid; i < valid_n; i += kSortThreads) {
            const uint32_t k = s_keys[i];
            const uint32_t gpos = s_out[(k >> shift) & MASK] + i;
            if (gpos < n) {  // always true unless a wait on the tree timed out (status already set)
                keys_out[gpos] = k;
                vals_out[gpos] = s_vals[i];
                if (ranges) {
                    // last pass: the keys of one tile are contiguous in the CTA's local order (one digit
                    // run, sorted by the lower bits), so the ends of each run of a tile give its range
                    // bounds (tile_ranges.wgsl:7-34), combined over the CTAs by min / max
                    const uint32_t tile = k >> 16u;
                    if (tile < tiles) {
                        if (i == 0u || (s_keys[i - 1u] >> 16u) != tile) atomicMin(&ranges[2u * tile], gpos);
                        if (i + 1u == valid_n || (s_keys[i + 1u] >> 16u) != tile) atomicMax(&ranges[2u * tile + 1u], gpos + 1u);
                    }
                }
            }
        }
    }
}

// ---- tile order: heaviest tiles first ----------------------------------------------------------------
// The raster CTAs take their tiles from `order` (CTA i renders tile order[i]); CTAs start roughly in
// index order, so listing the tiles by decreasing range length keeps the long tiles from forming the
// tail of the launch. Lengths are binned (four bins per octave, 64 bins, longest first) and placed by
// a counting sort; the order inside a bin is whatever the atomics give and changes no output, since
// every tile is rendered exactly once either way.
__device__ __forceinline__ uint32_t order_bin(uint32_t len) {
    const uint32_t v = len + 1u;
    const uint32_t msb = 31u - __clz(v);
    const uint32_t sub = msb >= 2u ? (v >> (msb - 2u)) & 3u : (v << (2u - msb)) & 3u;
    const uint32_t b = msb * 4u + sub;
    return 63u - min(b, 63u);
}

// Two kernels over slices of kOrderSlice tiles (one CTA each): k_tile_bins writes each slice's bin
// counts to row `slice` of a [slices x 64] table; k_tile_place gives every bin its global base (the
// bins before it over all slices, longest first) plus the same bin's count in earlier slices, and
// places the slice's tiles from there.
constexpr uint32_t kOrderThreads = 256;
constexpr uint32_t kOrderPer = 4;                                  // tiles per thread
constexpr uint32_t kOrderSlice = kOrderThreads * kOrderPer;        // tiles per CTA

// the bins of the calling thread's kOrderPer tiles of slice `slice` (64 for tiles past the end);
// all loads are issued before any is used
__device__ __forceinline__ void slice_bins(const uint32_t* __restrict__ ranges, uint32_t tiles, uint32_t slice,
                                           uint32_t b[kOrderPer]) {
    uint2 r[kOrderPer];
#pragma unroll
    for (uint32_t k = 0; k < kOrderPer; ++k) {
        const uint32_t t = slice * kOrderSlice + k * kOrderThreads + threadIdx.x;
        r[k] = t < tiles ? reinterpret_cast<const uint2*>(ranges)[t] : make_uint2(0u, 0u);
    }
#pragma unroll
    for (uint32_t k = 0; k < kOrderPer; ++k) {
        const uint32_t t = slice * kOrderSlice + k * kOrderThreads + threadIdx.x;
        b[k] = t < tiles ? order_bin(r[k].y > r[k].x ? r[k].y - r[k].x : 0u) : 64u;
    }
}

__global__ void __launch_bounds__(kOrderThreads) k_tile_bins(const uint32_t* __restrict__ ranges, uint32_t tiles,
                                                             uint32_t* __restrict__ slice_hist) {
    pdl_wait();
    __shared__ uint32_t s_bin[65];
    if (threadIdx.x < 65u) s_bin[threadIdx.x] = 0u;
    __syncthreads();
    uint32_t b[kOrderPer];
    slice_bins(ranges, tiles, blockIdx.x, b);
#pragma unroll
    for (uint32_t k = 0; k < kOrderPer; ++k) atomicAdd(&s_bin[b[k]], 1u);
    __syncthreads();
    if (threadIdx.x < 64u) slice_hist[blockIdx.x * 64u + threadIdx.x] = s_bin[threadIdx.x];
}

__global__ void __launch_bounds__(kOrderThreads) k_tile_place(uint32_t* __restrict__ ranges, uint32_t tiles,
                                                              const uint32_t* __restrict__ slice_hist,
                                                              uint32_t* __restrict__ order, uint32_t* status) {
    pdl_wait();
    __shared__ uint32_t s_incl[64];
    __shared__ uint32_t s_base[64];
    const uint32_t tid = threadIdx.x, slices = gridDim.x;
    uint32_t b[kOrderPer];
    slice_bins(ranges, tiles, blockIdx.x, b);  // in flight while the table is summed
    uint32_t total = 0, before = 0, incl = 0;
    if (tid < 64u) {  // warps 0 and 1: one bin per thread
        for (uint32_t s = 0; s < slices; ++s) {
            const uint32_t h = slice_hist[s * 64u + tid];
            total += h;
            before += s < blockIdx.x ? h : 0u;
        }
        incl = total;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if ((tid & 31u) >= (uint32_t)o) incl += t;
        }
        s_incl[tid] = incl;
    }
    __syncthreads();
    if (tid < 64u) s_base[tid] = (tid >= 32u ? s_incl[31] : 0u) + incl - total + before;
    __syncthreads();
#pragma unroll
    for (uint32_t k = 0; k < kOrderPer; ++k) {
        const uint32_t t = blockIdx.x * kOrderSlice + k * kOrderThreads + tid;
        if (t < tiles) {
            const uint32_t at = atomicAdd(&s_base[b[k]], 1u);
            if (GS_IN_BOUNDS(at, tiles, status)) order[at] = t;
            // bin 63 is length 0: a tile the last sort pass left at its cleared bounds
            if (b[k] == 63u) reinterpret_cast<uint2*>(ranges)[t] = make_uint2(0u, 0u);
        }
    }
}

// canary check: one CTA per buffer, one word of each pad per thread
__global__ void k_check_canaries(CanaryList list, uint32_t* status) {
    const uint32_t b = blockIdx.x;
    if (b >= list.count) return;
    bool bad = false;
    for (uint32_t w = threadIdx.x; w < kCanaryBytes / 4u; w += blockDim.x)
        bad |= list.head[b][w] != kCanaryWord || list.tail[b][w] != kCanaryWord;
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(status, kDevCanary);
}

// SM count of the current device (contexts of one process share a GPU model; read once, and from
// any thread).
int sm_count() {
    static std::atomic<int> cached{0};
    int v = cached.load(std::memory_order_relaxed);
    if (v == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        v = v > 0 ? v : 1;
        cached.store(v, std::memory_order_relaxed);
    }
    return v;
}

}  // namespace

void launch_frame_begin_multi(const MultiViewFrames& mv, cudaStream_t s) {
    uint32_t quads = 0;
    for (uint32_t v = 0; v < mv.count; ++v) quads = std::max(quads, mv.range_words[v] / 4u);
    const uint32_t grid = std::max(1u, std::min(64u, (quads + 255u) / 256u));
    launch_pdl(k_frame_begin_multi, dim3(grid, mv.count), dim3(256), s, mv);
}

void launch_frame_begin(FrameCtl* ctl, uint64_t* flags, uint32_t flag_words, cudaStream_t s, uint32_t* ranges,
                        uint32_t range_words) {
    // ranges come from cudaMalloc (16-byte aligned); one 16-byte store per thread, up to 64 CTAs
    const uint32_t quads = range_words / 4u;
    const uint32_t grid = std::max(1u, std::min(64u, (quads + 255u) / 256u));
    launch_pdl(k_frame_begin, dim3(grid), dim3(256), s, ctl, ranges, range_words, flags, flag_words);
}

void launch_scan_emit(const uint32_t* counts, const uint4* meta, uint32_t n, uint32_t tiles_x, uint32_t max_instance,
                      uint32_t digit_bits, uint32_t passes, uint32_t* offsets, uint32_t* keys, uint32_t* vals,
                      FrameCtl* ctl, uint64_t* flags, uint32_t slot, cudaStream_t s) {
    const uint32_t parts = (n + 1u + kScanPartition - 1u) / kScanPartition;
    launch_pdl(k_scan_emit, dim3(parts), dim3(kScanThreads), s, counts, meta, n, tiles_x, max_instance, digit_bits,
               passes, offsets, keys, vals, ctl, flags, slot);
}

void launch_exclusive_scan(uint32_t* data, uint32_t n, uint32_t* total_dev, FrameCtl* ctl, uint64_t* flags,
                           uint32_t slot, cudaStream_t s, uint32_t grid) {
    const uint32_t parts = n == 0 ? 1u : (n + kScanPartition - 1u) / kScanPartition;
    k_exclusive_scan<<<grid ? min(grid, parts) : parts, kScanThreads, 0, s>>>(data, n, total_dev, ctl, flags, slot);
}

void launch_digit_hist(const uint32_t* keys, uint32_t n, uint32_t digit_bits, uint32_t key_bits, uint32_t* hist,
                       cudaStream_t s) {
    uint32_t blocks = (n + 1023u) / 1024u;
    const uint32_t cap = (uint32_t)sm_count() * 4u;
    if (blocks > cap) blocks = cap;
    if (blocks == 0) blocks = 1;
    k_digit_hist<<<blocks, 256, 0, s>>>(keys, n, digit_bits, key_bits, hist);
}

void configure_sort_kernels() {
    // the largest shared-memory carveout lets more onesweep CTAs (up to 44 KB each) share an SM
    cudaFuncSetAttribute(k_onesweep<4, 8, 0>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    cudaFuncSetAttribute(k_onesweep<4, 16, 0>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    cudaFuncSetAttribute(k_onesweep<8, 8, 0>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    cudaFuncSetAttribute(k_onesweep<8, 8, 2>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    cudaFuncSetAttribute(k_onesweep<8, 8, 3>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    cudaFuncSetAttribute(k_onesweep<8, 8, 4>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    cudaFuncSetAttribute(k_onesweep<8, 16, 0>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    cudaFuncSetAttribute(k_onesweep<8, 16, 2>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    cudaFuncSetAttribute(k_onesweep<8, 16, 3>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    cudaFuncSetAttribute(k_onesweep<8, 16, 4>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
}

void launch_onesweep(uint32_t digit_bits, const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                     uint32_t* vals_out, const uint32_t* n_dev, uint32_t n_host, uint32_t max_n, uint32_t shift,
                     uint32_t dmask, const uint32_t* hist, FrameCtl* ctl, uint64_t* flags, uint32_t slot,
                     int grid_cap, cudaStream_t s, uint32_t block, uint32_t split, bool early, uint32_t* ranges,
                     uint32_t tiles) {
    const bool small = block == kSortPartitionMin;
    const uint32_t part = small ? kSortPartitionMin : kSortPartition;
    uint32_t parts = (max_n + part - 1u) / part;
    const uint32_t cap = grid_cap > 0 ? (uint32_t)grid_cap : (uint32_t)sm_count() * 4u;
    if (parts > cap) parts = cap;
    if (parts == 0) parts = 1;
#define GS_ONESWEEP(B, I, S)                                                                                      \
    launch_pdl(k_onesweep<B, I, S>, dim3(parts), dim3(kSortThreads), s, keys_in, vals_in, keys_out, vals_out, n_dev, \
               n_host, shift, dmask, hist, ctl, flags, slot, early ? 1u : 0u, ranges, tiles)
#define GS_ONESWEEP_SPLIT(I)                             \
    switch (split) {                                     \
        case 2: GS_ONESWEEP(8, I, 2); break;             \
        case 3: GS_ONESWEEP(8, I, 3); break;             \
        case 4: GS_ONESWEEP(8, I, 4); break;             \
        default: GS_ONESWEEP(8, I, 0); break;            \
    }
    if (digit_bits == 4) {  // 16 digit values at most: the plain match
        if (small) GS_ONESWEEP(4, 8, 0); else GS_ONESWEEP(4, 16, 0);
    } else {
        if (small) GS_ONESWEEP_SPLIT(8) else GS_ONESWEEP_SPLIT(16)
    }
#undef GS_ONESWEEP_SPLIT
#undef GS_ONESWEEP
}

void launch_check_canaries(const CanaryList& list, uint32_t* status, cudaStream_t s) {
    if (list.count) k_check_canaries<<<list.count, kCanaryBytes / 4u, 0, s>>>(list, status);
}

uint32_t tile_order_slices(uint32_t tiles) { return (tiles + kOrderSlice - 1u) / kOrderSlice; }

void launch_tile_order(uint32_t* ranges, uint32_t tiles, uint32_t* slice_hist, uint32_t* order, uint32_t* status,
                       cudaStream_t s) {
    const uint32_t slices = std::max(1u, tile_order_slices(tiles));
    launch_pdl(k_tile_bins, dim3(slices), dim3(kOrderThreads), s, ranges, tiles, slice_hist);
    launch_pdl(k_tile_place, dim3(slices), dim3(kOrderThreads), s, ranges, tiles, (const uint32_t*)slice_hist, order,
               status);
}


}  // namespace gs
