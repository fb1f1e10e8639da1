// Stable LSD key/value radix sort, 8-bit digits, one sweep per digit.
//
// Replaces the reference's vrdxCmdSortKeyValue (upsweep -> spine ->
// downsweep per pass, external/vulkan_radix_sort/vk_radix_sort.h:2598-2755)
// with a single-sweep scheme after Adinets & Merrill ("Onesweep", 2022):
//   1. one histogram kernel reads the keys once and builds the 256-bin digit
//      histogram of every pass (the global digit bases);
//   2. per pass, one kernel of 512-thread CTAs, two resident per SM: each takes
//      the next tile from a ticket counter, has L2 prefetch a tile half a wave
//      ahead, ranks its keys with warp ballots
//      (stable: keys are ranked in input order), publishes its per-digit
//      counts, stages the tile in shared memory in digit order, resolves the
//      global digit offsets with a bounded decoupled look-back over earlier
//      tiles and writes keys and values out in coalesced runs.
// Sized for a frame's wavefronts (a few million keys, all of it resident in
// L2): tiles of 8 or 14-16 keys per thread make such a pass one wave of
// about two tiles per SM, and the look-back reads 8 predecessors per L2
// round trip with a cheap test for the common round of published aggregates;
// staging the tile before the look-back overlaps that wait with useful work.
// Ping-pong between the caller's buffers and scratch; after an even number
// of passes the result is back in the caller's buffers (as in the reference),
// after an odd number it is copied back.
#include <algorithm>
#include <utility>

#include "common.cuh"
#include "stages.cuh"

namespace wfpt {

cudaError_t status_sort(uint32_t* out) { return read_and_clear_status(out); }

constexpr int kSortThreads = 512;
constexpr int kSortWarps = kSortThreads / 32;
// Resident pass CTAs per SM (registers: 2 x 512 threads x 64; shared
// memory: two large-tile CTAs fit in an SM's 228 KB).  Two CTAs let one
// tile's ranking overlap the other's scatter and look-back wait; one
// 1024-thread CTA per SM was 17-18 % slower on 2^24-2^26 keys.
constexpr int kSortCtasPerSm = 2;
constexpr int kRadix = 256;
constexpr int kHistBlock = 256;
constexpr uint32_t kLbAggregate = 1u << 30;
constexpr uint32_t kLbPrefix = 2u << 30;
constexpr uint32_t kLbValue = (1u << 30) - 1u;
// Predecessors read per look-back round trip.  With the all-aggregates fast
// path below, 8 measured 1-4 % faster per sort than 16 at 16.8M-67M pairs
// and equal at 2.07M (24 and 32 slower): a round is bound by the owner
// warps' instructions as much as by the L2 round trip.
constexpr int kLbChunk = 8;

// Keys per thread of the tile variants (tile = 512 * KPT keys).  The
// extra-large variant serves sorts of more than two waves of large tiles:
// 20 keys per thread for 32-bit keys (10 % faster than 16 on 2^26 keys).
// For 64-bit keys it is the large tile (15 keys per thread measured 2-4 %
// slower on 2^24-2^26 keys; 14 is close to the most that leaves room for
// two CTAs per SM).
constexpr int kKptSmall32 = 8, kKptLarge32 = 16, kKptXLarge32 = 20;
constexpr int kKptSmall64 = 8, kKptLarge64 = 14, kKptXLarge64 = kKptLarge64;

// Digit mask of pass p with db-bit digits: the top pass keeps only the
// bits below key_bits.
__host__ __device__ __forceinline__ uint32_t pass_mask(int key_bits, int p, int db = 8) {
    int bits = key_bits - db * p;
    return bits >= db ? ((1u << db) - 1u) : ((1u << bits) - 1u);
}
__device__ __forceinline__ uint32_t digit_of(uint32_t k, int shift, uint32_t dmask) { return (k >> shift) & dmask; }
__device__ __forceinline__ uint32_t digit_of(uint64_t k, int shift, uint32_t dmask) { return (uint32_t)(k >> shift) & dmask; }

// Lanes of the warp whose tested bit equals this lane's (`bit` is the
// lane's key digit masked to one bit): the ballot of the bit, complemented
// under the lane's own predicate when the bit is clear.  Written in PTX so
// that the predicate of the vote also selects the complement (measured 4-8 %
// faster per sort than a branch-free select in C++).
__device__ __forceinline__ uint32_t same_bit_lanes(uint32_t bit) {
    uint32_t m;
    asm("{\n\t.reg .pred q;\n\t"
        "setp.ne.u32 q, %1, 0;\n\t"
        "vote.sync.ballot.b32 %0, q, 0xffffffff;\n\t"
        "@!q not.b32 %0, %0;\n\t}"
        : "=r"(m)
        : "r"(bit));
    return m;
}

// Exclusive scan of one value per thread over the whole block (blockDim.x =
// 32 * W); *total receives the block sum.  Every thread must call it.
template <int W>
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* s_warp, uint32_t* total) {
    uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    uint32_t off = 0, sum = 0;
#pragma unroll
    for (int w = 0; w < W; ++w) {
        uint32_t c = s_warp[w];
        if (w < (int)warp) off += c;
        sum += c;
    }
    __syncthreads();
    *total = sum;
    return off + x - v;
}

// Byte p of a key (digit of pass p before the top-pass mask).
__device__ __forceinline__ uint32_t key_byte(uint32_t k, int p) { return p < 4 ? (k >> (8 * p)) & 0xFFu : 0u; }
__device__ __forceinline__ uint32_t key_byte(uint64_t k, int p) {
    return p < 4 ? ((uint32_t)k >> (8 * p)) & 0xFFu : ((uint32_t)(k >> 32) >> (8 * (p - 4))) & 0xFFu;
}

// Programmatic dependent launch between the sort's kernels.  A pass kernel
// is launched with programmatic stream serialisation: its CTAs may start
// once every CTA of the previous kernel has started (or exited) and run
// their prologue (ticket, clearing the counters) while the previous kernel
// finishes; wait_for_previous_grid() then blocks until that kernel has
// completed and its writes are visible.  Nothing the previous kernel writes
// is read before the wait.  At a frame's sort size (one wave of tiles per
// pass) this hides the launch gap and the ticket round trip of every pass:
// 10 % faster sorts of 2.07M u64 pairs, 7 % at 16.8M, 2.5 % at 67M.
__device__ __forceinline__ void allow_dependent_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void wait_for_previous_grid() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename Kernel, typename... Args>
static cudaError_t launch_dependent(Kernel kernel, unsigned grid, unsigned block, size_t smem, cudaStream_t s,
                                    Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// Histogram of every pass's digit over the first `count` keys: PASSES is a
// template parameter so that the digit extraction unrolls into constant
// byte selects; each thread issues the loads of 8 keys before their
// shared-memory atomics.
template <typename K, int PASSES>
__global__ void __launch_bounds__(kHistBlock) k_sort_hist(const K* __restrict__ keys, uint32_t n,
                                                           const uint32_t* __restrict__ n_dev, uint32_t top_mask,
                                                           uint32_t* __restrict__ hist) {
    constexpr int U = 8;
    __shared__ uint32_t s_h[PASSES * kRadix];
    // Every CTA of this grid has started: the first pass may launch its
    // CTAs into the slots this grid frees (they wait for its completion).
    allow_dependent_launch();
    for (int i = threadIdx.x; i < PASSES * kRadix; i += kHistBlock) s_h[i] = 0;
    __syncthreads();
    const uint32_t count = load_count(n, n_dev);
    const uint32_t step = gridDim.x * kHistBlock * U;
    for (uint32_t i0 = blockIdx.x * kHistBlock * U + threadIdx.x; i0 < count; i0 += step) {
        K kk[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            uint32_t i = i0 + u * kHistBlock;
            kk[u] = i < count ? keys[i] : (K)0;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (i0 + u * kHistBlock < count) {
#pragma unroll
                for (int p = 0; p < PASSES; ++p) {
                    uint32_t d = key_byte(kk[u], p);
                    if (p == PASSES - 1) d &= top_mask;
                    atomicAdd(&s_h[p * kRadix + d], 1u);
                }
            }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < PASSES * kRadix; i += kHistBlock) {
        uint32_t c = s_h[i];
        if (c) atomicAdd(&hist[i], c);
    }
}

// The same histograms for large sorts of wide keys (kHistColsMin keys and
// more, five passes or more), with the atomics spread so that no two lanes
// of a warp meet in a shared-memory bank: every lane owns a column of 16-bit counter pairs (two adjacent
// digits per word, the word of digit d of pass p at row p * 128 + d / 2,
// column lane), shared by the same lane of all 32 warps of a 1024-thread
// CTA (one per SM, PASSES x 16 KB of shared memory).  At the end each CTA
// sums the 32 columns of every counter and adds it to the global
// histogram.  A counter never passes 65,535: a lane handles at most
// kHistColsMaxIters x 8 keys, so a column at most 32 times that (the grid
// grows with n to keep it so).  15 % faster than k_sort_hist on 2^26 u64
// keys (0.172 against 0.202 ms, A/B harness): the conflicts of random digits
// had cost about that much of the atomics' throughput.  Whole u64 sorts: 1.2 %
// faster at 2^26 pairs (3.249 -> 3.211 ms), 1.0 % at 2^25, 0.7 % at 2^24.
// With four passes or fewer (u32 keys) the histogram kernel is bound by
// reading the keys rather than by its atomics, and the columns' set-up and
// reduction made 2^24-pair sorts 1 % slower: those keep k_sort_hist.
constexpr int kHistColsBlock = 1024;
constexpr uint32_t kHistColsMin = 1u << 24;
constexpr uint32_t kHistColsMaxIters = 255;  // 255 * 8 * 32 = 65,280 per counter at most

template <typename K, int PASSES>
__global__ void __launch_bounds__(kHistColsBlock) k_sort_hist_cols(const K* __restrict__ keys, uint32_t n,
                                                                   const uint32_t* __restrict__ n_dev,
                                                                   uint32_t top_mask, uint32_t* __restrict__ hist) {
    constexpr int U = 8;
    constexpr int kWords = PASSES * (kRadix / 2) * 32;
    extern __shared__ uint32_t s_col[];  // [PASSES * 128][32]
    allow_dependent_launch();
    for (int i = threadIdx.x; i < kWords; i += kHistColsBlock) s_col[i] = 0;
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t count = load_count(n, n_dev);
    const uint32_t step = gridDim.x * kHistColsBlock * U;
    for (uint32_t i0 = blockIdx.x * kHistColsBlock * U + threadIdx.x; i0 < count; i0 += step) {
        K kk[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            uint32_t i = i0 + u * kHistColsBlock;
            kk[u] = i < count ? keys[i] : (K)0;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (i0 + u * kHistColsBlock < count) {
#pragma unroll
                for (int p = 0; p < PASSES; ++p) {
                    uint32_t d = key_byte(kk[u], p);
                    if (p == PASSES - 1) d &= top_mask;
                    atomicAdd(&s_col[(p * (kRadix / 2) + (d >> 1)) * 32 + lane], 1u << ((d & 1u) * 16u));
                }
            }
        }
    }
    __syncthreads();
    // Counter c (pass c / 256, digit c % 256): the sum of its 32 columns,
    // read from a rotated start so that a warp's 32 counters hit 32 banks.
    for (int c = threadIdx.x; c < PASSES * kRadix; c += kHistColsBlock) {
        const uint32_t* row = s_col + (c >> 1) * 32;
        const uint32_t sh = (uint32_t)(c & 1) * 16u;
        uint32_t sum = 0;
#pragma unroll 8
        for (int l = 0; l < 32; ++l) sum += (row[(l + c) & 31] >> sh) & 0xFFFFu;
        if (sum) atomicAdd(&hist[c], sum);
    }
}

template <typename K, int PASSES>
static cudaError_t opt_in_hist_cols() {
    return cudaFuncSetAttribute(k_sort_hist_cols<K, PASSES>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                PASSES * (kRadix / 2) * 32 * 4);
}

template <typename K>
static void launch_hist(const K* keys, uint32_t n, const uint32_t* n_dev, int passes, int key_bits,
                        uint32_t* hist, unsigned grid, unsigned sms, cudaStream_t s) {
    const uint32_t top = pass_mask(key_bits, passes - 1);
    if constexpr (sizeof(K) == 8) {
        if (n >= kHistColsMin && passes > 4) {
            // One CTA per SM, more when a lane would otherwise count more
            // than kHistColsMaxIters rounds of 8 keys.
            const size_t per_cta = (size_t)kHistColsMaxIters * 8 * kHistColsBlock;
            const unsigned cgrid = (unsigned)std::max<size_t>((size_t)sms, ((size_t)n + per_cta - 1) / per_cta);
            const size_t smem = (size_t)passes * (kRadix / 2) * 32 * 4;
            switch (passes) {
#define WFPT_HIST_COLS(P)                                                                              \
    case P:                                                                                            \
        k_sort_hist_cols<K, P><<<cgrid, kHistColsBlock, smem, s>>>(keys, n, n_dev, top, hist);         \
        return;
                WFPT_HIST_COLS(5) WFPT_HIST_COLS(6) WFPT_HIST_COLS(7) WFPT_HIST_COLS(8)
#undef WFPT_HIST_COLS
                default: return;
            }
        }
    }
    switch (passes) {
#define WFPT_HIST(P)                                                                                   \
    case P:                                                                                            \
        k_sort_hist<K, P><<<grid, kHistBlock, 0, s>>>(keys, n, n_dev, top, hist);                      \
        break;
        WFPT_HIST(1) WFPT_HIST(2) WFPT_HIST(3) WFPT_HIST(4) WFPT_HIST(5) WFPT_HIST(6) WFPT_HIST(7) WFPT_HIST(8)
#undef WFPT_HIST
        default: break;
    }
}

// Bulk prefetch into L2 of `count` keys and values (cp.async.bulk.prefetch:
// one instruction per array, 16-byte aligned start and size).  Arrays that
// are not 16-byte aligned are skipped; the loads then go to DRAM as usual.
template <typename K>
__device__ __forceinline__ void prefetch_l2(const K* keys, const uint32_t* vals, uint32_t count) {
    const uint32_t kb = count * (uint32_t)sizeof(K), vb = count * 4u;
    if (((reinterpret_cast<uintptr_t>(keys) | reinterpret_cast<uintptr_t>(vals) | kb | vb) & 15u) != 0) return;
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(keys), "r"(kb) : "memory");
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(vals), "r"(vb) : "memory");
}

// One tile of a digit pass (below).  FULL: the tile holds TILE keys, so
// the per-key bounds checks of the last, partial tile drop out.
template <typename K, int KPT, int DB, bool FULL>
__device__ __forceinline__ void onesweep_tile(const K* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
                                              K* __restrict__ keys_out, uint32_t* __restrict__ vals_out,
                                              uint32_t count, uint32_t tile, int shift, uint32_t dmask,
                                              const uint32_t* __restrict__ hist, uint32_t* __restrict__ lookback,
                                              int nibble, unsigned char* smem, uint32_t* s_scan) {
    constexpr uint32_t TILE = kSortThreads * KPT;
    constexpr int kRadix = 1 << DB;
    K* s_keys = reinterpret_cast<K*>(smem);
    uint32_t* s_vals = reinterpret_cast<uint32_t*>(s_keys + TILE);
    uint32_t* s_hist = s_vals + TILE;  // [warp][digit]
    uint32_t* s_base = s_hist + kSortWarps * kRadix;
    uint32_t* s_loc = s_base + kRadix;

    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lt_mask = (1u << lane) - 1u;
    const uint32_t base = tile * TILE + warp * 32 * KPT + lane;

    K key[KPT];
    uint32_t rank[KPT];
#pragma unroll
    for (int k = 0; k < KPT; ++k) {
        uint32_t i = base + k * 32;
        key[k] = (FULL || i < count) ? keys_in[i] : (K)0;
    }
    uint32_t* my_hist = s_hist + warp * kRadix;
    // Warp-level stable ranking: keys are visited in input order (k, lane).
#pragma unroll
    for (int k = 0; k < KPT; ++k) {
        const bool ok = FULL || (base + k * 32) < count;
        uint32_t d = digit_of(key[k], shift, dmask);
        uint32_t peers = FULL ? 0xffffffffu : __ballot_sync(0xffffffffu, ok);
#pragma unroll
        for (int b = 0; b < DB; ++b) peers &= same_bit_lanes(d & (1u << b));
        uint32_t before = peers & lt_mask;
        uint32_t pre = ok ? my_hist[d] : 0u;
        __syncwarp();
        if (ok && before == 0u) my_hist[d] = pre + __popc(peers);
        __syncwarp();
        rank[k] = pre + __popc(before);
    }
    __syncthreads();

    // Threads 0..RADIX-1 own one digit each: warp-exclusive prefixes and
    // the tile's count of that digit.
    const bool owner = threadIdx.x < kRadix;
    const uint32_t d = threadIdx.x & (kRadix - 1);
    uint32_t run = 0;
    if (owner) {
#pragma unroll 8
        for (int w = 0; w < kSortWarps; ++w) {
            uint32_t c = s_hist[w * kRadix + d];
            s_hist[w * kRadix + d] = run;
            run += c;
        }
    }
    uint32_t tile_total;
    const uint32_t loc = block_exclusive_scan<kSortWarps>(owner ? run : 0u, s_scan, &tile_total);
    // Publish this tile's counts (tile 0: its inclusive prefix, from the
    // global histogram) before staging, so that successors can proceed.
    uint32_t excl = 0;
    if (tile == 0) {
        uint32_t total, cnt_d = 0;
        if (owner) {
            if (DB == 8) {
                cnt_d = hist[d];
            } else {
#pragma unroll
                for (uint32_t j = 0; j < 16; ++j) cnt_d += hist[nibble ? ((d << 4) | j) : ((j << 4) | d)];
            }
        }
        excl = block_exclusive_scan<kSortWarps>(cnt_d, s_scan, &total);
    }
    uint32_t* lb = lookback + (size_t)tile * kRadix + d;
    if (owner) {
        s_loc[d] = loc;
        atomicExch(lb, tile == 0 ? (kLbPrefix | (excl + run)) : (kLbAggregate | run));
    }
    __syncthreads();

    // Stage the tile in digit order; values are read here, straight from
    // global memory into their sorted slot.
#pragma unroll
    for (int k = 0; k < KPT; ++k) {
        uint32_t i = base + k * 32;
        if (FULL || i < count) {
            uint32_t dk = digit_of(key[k], shift, dmask);
            uint32_t pos = s_loc[dk] + my_hist[dk] + rank[k];
            s_keys[pos] = key[k];
            s_vals[pos] = vals_in[i];
        }
    }

    // Decoupled look-back for digit d: walk back over predecessors, kLbChunk
    // of them per round trip with independent loads; stop at the first
    // inclusive prefix, wait (bounded) on an entry that is not published yet.
    if (owner && tile != 0) {
        int32_t j = (int32_t)tile - 1;
        uint32_t spins = 0;
        bool done = false;
        while (!done && j >= 0) {
            uint32_t st[kLbChunk];
#pragma unroll
            for (int q = 0; q < kLbChunk; ++q)
                st[q] = (j - q >= 0) ? *((volatile uint32_t*)(lookback + (size_t)(j - q) * kRadix + d))
                                     : uint32_t(kLbPrefix);
            // Fast path: every entry a published aggregate (flag bit 30 set
            // in all of them; a prefix has bit 31 alone, an unpublished entry
            // neither).  Their raw sum minus the flags is the sum of the
            // counts, so the round costs an AND and an add per entry instead
            // of the sequential scan (5-9 % faster sorts at the frame's 2.07M
            // pairs, where most rounds are of this kind).
            {
                uint32_t all = 0xFFFFFFFFu, raw = 0u;
#pragma unroll
                for (int q = 0; q < kLbChunk; ++q) {
                    all &= st[q];
                    raw += st[q];
                }
                if (all & kLbAggregate) {
                    excl += raw - (uint32_t)kLbChunk * kLbAggregate;
                    j -= kLbChunk;
                    continue;
                }
            }
            int used = 0;
#pragma unroll
            for (int q = 0; q < kLbChunk; ++q) {
                if (done || used < q) continue;  // stopped earlier in this chunk
                uint32_t flag = st[q] & ~kLbValue;
                if (flag == 0u) continue;  // not published: re-read from here
                excl += st[q] & kLbValue;
                used = q + 1;
                if (flag == kLbPrefix) done = true;
            }
            j -= used;
            if (!done && used < kLbChunk && j >= 0) {
                if (++spins > kSpinLimit) {
                    raise_status(kErrTimeout);
                    break;
                }
                __nanosleep(32);
            }
        }
        atomicExch(lb, kLbPrefix | (excl + run));
    }
    if (owner) s_base[d] = excl - loc;
    __syncthreads();

    const uint32_t tile_count = FULL ? TILE : min(TILE, count - tile * TILE);
#pragma unroll 2
    for (uint32_t j = threadIdx.x; j < tile_count; j += kSortThreads) {
        K kk = s_keys[j];
        uint32_t g = s_base[digit_of(kk, shift, dmask)] + j;
        if (g < count) {  // only fails after a look-back timeout
            // Streaming stores: the output is next read by the following
            // pass, after far more than L2 holds has gone through it.
            __stcs(keys_out + g, kk);
            __stcs(vals_out + g, s_vals[j]);
        } else {
            raise_status(kErrBounds);
        }
    }
}

// One digit pass with DB-bit digits (RADIX = 2^DB bins).  Dynamic shared
// memory: TILE keys, TILE values, kSortWarps*RADIX per-warp digit
// counters, RADIX global bases, RADIX local offsets.  hist is the byte
// histogram (k_sort_hist) of this pass's byte; with 4-bit digits a digit's
// count is the sum of the 16 byte bins sharing that nibble (nibble 0: low
// nibble of the byte, 1: high nibble).  The CTA that draws tile t asks L2
// for the keys and values of tile t + lead (half the resident CTAs ahead:
// the tile that starts about half a tile's lifetime later), so that a
// tile's loads find their data in L2 instead of waiting on DRAM.
template <typename K, int KPT, int DB>
__global__ void __launch_bounds__(kSortThreads, kSortCtasPerSm) k_onesweep(const K* __restrict__ keys_in,
                                                              const uint32_t* __restrict__ vals_in,
                                                              K* __restrict__ keys_out,
                                                              uint32_t* __restrict__ vals_out, uint32_t n,
                                                              const uint32_t* __restrict__ n_dev, int shift,
                                                              uint32_t dmask, const uint32_t* __restrict__ hist,
                                                              uint32_t* __restrict__ lookback,
                                                              uint32_t* __restrict__ ticket, int nibble,
                                                              uint32_t lead) {
    constexpr uint32_t TILE = kSortThreads * KPT;
    constexpr int kRadix = 1 << DB;
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t* s_hist = reinterpret_cast<uint32_t*>(smem + (size_t)TILE * (sizeof(K) + 4));
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_scan[kSortWarps];

    // Prologue that reads nothing the previous kernel writes (the tickets
    // and look-back states of this pass were cleared before the sort began).
    uint32_t t = 0;
    if (threadIdx.x == 0) t = atomicAdd(ticket, 1u);
    for (int i = threadIdx.x; i < kSortWarps * kRadix; i += kSortThreads) s_hist[i] = 0;
    allow_dependent_launch();
    wait_for_previous_grid();
    const uint32_t count = load_count(n, n_dev);
    const uint32_t ntiles = (count + TILE - 1) / TILE;
    if (threadIdx.x == 0) {
        s_tile = t;
        const uint32_t ahead = t + lead;
        if (lead != 0 && ahead > t && (size_t)(ahead + 1) * TILE <= count)
            prefetch_l2(keys_in + (size_t)ahead * TILE, vals_in + (size_t)ahead * TILE, TILE);
    }
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile >= ntiles) return;
    if ((size_t)(tile + 1) * TILE <= count)
        onesweep_tile<K, KPT, DB, true>(keys_in, vals_in, keys_out, vals_out, count, tile, shift, dmask, hist,
                                        lookback, nibble, smem, s_scan);
    else
        onesweep_tile<K, KPT, DB, false>(keys_in, vals_in, keys_out, vals_out, count, tile, shift, dmask, hist,
                                         lookback, nibble, smem, s_scan);
}

// After an odd number of passes: move the first `count` pairs back into the
// caller's buffers (elements past the device-side count stay untouched).
template <typename K>
__global__ void k_copy_back(const K* __restrict__ ks, const uint32_t* __restrict__ vs, K* __restrict__ kd,
                            uint32_t* __restrict__ vd, uint32_t n, const uint32_t* __restrict__ n_dev) {
    uint32_t count = load_count(n, n_dev);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        kd[i] = ks[i];
        vd[i] = vs[i];
    }
}

static inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

template <typename K, int KPT, int DB>
static size_t onesweep_smem() {
    return (size_t)kSortThreads * KPT * (sizeof(K) + 4) + (size_t)(kSortWarps + 2) * (1u << DB) * 4;
}

template <typename K, int KPT, int DB>
static cudaError_t opt_in_smem() {
    return cudaFuncSetAttribute(k_onesweep<K, KPT, DB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)onesweep_smem<K, KPT, DB>());
}

static int g_num_sms = 0;

// Opts the pass kernels into their dynamic shared memory and reads the SM
// count once (host calls that must not run inside a stream capture; the
// renderer calls this before capturing a frame graph).
cudaError_t sort_prepare() {
    if (g_num_sms != 0) return cudaSuccess;
    cudaError_t e = opt_in_smem<uint32_t, kKptSmall32, 8>();
    if (e == cudaSuccess) e = opt_in_smem<uint32_t, kKptLarge32, 8>();
    if (e == cudaSuccess) e = opt_in_smem<uint32_t, kKptXLarge32, 8>();
    if (e == cudaSuccess) e = opt_in_smem<uint32_t, kKptXLarge32, 4>();
    if (e == cudaSuccess) e = opt_in_smem<uint64_t, kKptSmall64, 8>();
    if (e == cudaSuccess) e = opt_in_smem<uint64_t, kKptLarge64, 8>();
    if (e == cudaSuccess) e = opt_in_smem<uint32_t, kKptSmall32, 4>();
    if (e == cudaSuccess) e = opt_in_smem<uint32_t, kKptLarge32, 4>();
    if (e == cudaSuccess) e = opt_in_smem<uint64_t, kKptSmall64, 4>();
    if (e == cudaSuccess) e = opt_in_smem<uint64_t, kKptLarge64, 4>();
    if (e == cudaSuccess) e = opt_in_hist_cols<uint64_t, 5>();
    if (e == cudaSuccess) e = opt_in_hist_cols<uint64_t, 6>();
    if (e == cudaSuccess) e = opt_in_hist_cols<uint64_t, 7>();
    if (e == cudaSuccess) e = opt_in_hist_cols<uint64_t, 8>();
    int dev = 0, sms = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) g_num_sms = sms > 0 ? sms : 1;
    return e;
}

// Tile variant: 0 = automatic, 1 = small, 2 = large, 3 = extra-large tiles
// (64-bit keys: the large ones).  Automatic takes the small tiles while they
// fit in one wave (two tiles per SM), the large ones while those fit in two
// waves (a frame-sized sort), and the extra-large ones beyond.
static int g_sort_tiles = 0;
void set_sort_tiles(int v) { g_sort_tiles = v < 0 ? 0 : (v > 3 ? 3 : v); }
int get_sort_tiles() { return g_sort_tiles; }

// Digit width: 8 (default) or 4 bits per pass (twice the passes, 16-bin
// ranking).
static int g_digit_bits = 8;
void set_sort_digit_bits(int v) { g_digit_bits = v == 4 ? 4 : 8; }
int get_sort_digit_bits() { return g_digit_bits; }

static int tile_variant(uint32_t n, bool wide) {
    if (g_sort_tiles != 0) return g_sort_tiles;
    const size_t slots = (size_t)g_num_sms * kSortCtasPerSm;
    const size_t small = (size_t)kSortThreads * (wide ? kKptSmall64 : kKptSmall32);
    const size_t large = (size_t)kSortThreads * (wide ? kKptLarge64 : kKptLarge32);
    if (((size_t)n + small - 1) / small <= slots) return 1;
    return ((size_t)n + large - 1) / large <= 2 * slots ? 2 : 3;
}

struct SortLayout {
    int passes;
    size_t key_bytes;
    size_t tiles;  // tiles of the small variant (the larger count)
    size_t off_ticket, off_hist, off_lookback, off_keys, off_vals, total;
};

static SortLayout sort_layout(uint32_t max_n, int key_bits) {
    SortLayout L;
    L.passes = (key_bits + 7) / 8;
    L.key_bytes = key_bits <= 32 ? 4 : 8;
    size_t tile = (size_t)kSortThreads * (key_bits <= 32 ? kKptSmall32 : kKptSmall64);
    L.tiles = std::max<size_t>(1, ((size_t)max_n + tile - 1) / tile);
    L.off_ticket = 0;
    L.off_hist = 256;
    L.off_lookback = L.off_hist + align256((size_t)L.passes * kRadix * 4);
    L.off_keys = L.off_lookback + align256((size_t)L.passes * L.tiles * kRadix * 4);
    L.off_vals = L.off_keys + align256((size_t)max_n * L.key_bytes);
    L.total = L.off_vals + align256((size_t)max_n * 4);
    return L;
}

size_t sort_scratch_bytes(uint32_t max_n, int key_bits) {
    if (key_bits < 1 || key_bits > 64) return 0;
    return sort_layout(max_n, key_bits).total;
}

// The layout is sized for 8-bit digits; 4-bit digits take at most twice the
// passes with 1/16 of the look-back entries per pass, and their global digit
// counts come from the same byte histograms.
template <typename K, int KPT, int DB>
static cudaError_t sort_passes(K* keys, uint32_t* values, uint32_t n, const uint32_t* n_dev, int key_bits,
                               const SortLayout& L, unsigned char* scratch, cudaStream_t s) {
    constexpr uint32_t TILE = kSortThreads * KPT;
    constexpr uint32_t RADIX = 1u << DB;
    const int passes = (key_bits + DB - 1) / DB;
    uint32_t* tickets = reinterpret_cast<uint32_t*>(scratch + L.off_ticket);
    uint32_t* hist = reinterpret_cast<uint32_t*>(scratch + L.off_hist);
    uint32_t* lookback = reinterpret_cast<uint32_t*>(scratch + L.off_lookback);
    K* alt_keys = reinterpret_cast<K*>(scratch + L.off_keys);
    uint32_t* alt_vals = reinterpret_cast<uint32_t*>(scratch + L.off_vals);
    const uint32_t tiles = (n + TILE - 1) / TILE;
    const size_t smem = onesweep_smem<K, KPT, DB>();
    // Prefetch distance in tiles: half the CTAs resident at once (measured
    // 3/8 to 5/8 of them equally good at 2^24-2^26 pairs; a whole wave
    // ahead was 6 % slower, two waves slower than no prefetch).
    const uint32_t lead = (uint32_t)(g_num_sms * kSortCtasPerSm / 2);
    cudaError_t e;
    K* src_k = keys;
    uint32_t* src_v = values;
    K* dst_k = alt_keys;
    uint32_t* dst_v = alt_vals;
    for (int p = 0; p < passes; ++p) {
        const int byte = DB == 8 ? p : p / 2;
        e = launch_dependent(k_onesweep<K, KPT, DB>, tiles, kSortThreads, smem, s, (const K*)src_k,
                             (const uint32_t*)src_v, dst_k, dst_v, n, n_dev, (int)(DB * p), pass_mask(key_bits, p, DB),
                             (const uint32_t*)(hist + byte * kRadix), lookback + (size_t)p * L.tiles * RADIX,
                             tickets + p, (int)(DB == 8 ? 0 : (p & 1)), lead);
        count_launch();
        if (e != cudaSuccess || (e = cudaGetLastError()) != cudaSuccess) return e;
        std::swap(src_k, dst_k);
        std::swap(src_v, dst_v);
    }
    if (passes & 1) {
        unsigned cgrid = (unsigned)std::min<size_t>(((size_t)n + 255) / 256, 152 * 16);
        k_copy_back<K><<<cgrid, 256, 0, s>>>(alt_keys, alt_vals, keys, values, n, n_dev);
        count_launch();
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

template <typename K>
static cudaError_t sort_impl(K* keys, uint32_t* values, uint32_t n, const uint32_t* n_dev, int key_bits,
                             unsigned char* scratch, cudaStream_t s) {
    SortLayout L = sort_layout(n, key_bits);
    cudaError_t e;
    if ((e = sort_prepare()) != cudaSuccess) return e;
    // Tickets, histograms and look-back states start at zero.
    if ((e = cudaMemsetAsync(scratch, 0, L.off_keys, s)) != cudaSuccess) return e;
    uint32_t* hist = reinterpret_cast<uint32_t*>(scratch + L.off_hist);
    unsigned hgrid = (unsigned)std::min<size_t>(((size_t)n + kHistBlock * 8 - 1) / (kHistBlock * 8),
                                                (size_t)g_num_sms * 8);
    if (hgrid == 0) hgrid = 1;
    launch_hist<K>(keys, n, n_dev, L.passes, key_bits, hist, hgrid, (unsigned)g_num_sms, s);
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    constexpr bool wide = sizeof(K) == 8;
    constexpr int small = wide ? kKptSmall64 : kKptSmall32, large = wide ? kKptLarge64 : kKptLarge32;
    constexpr int xlarge = wide ? kKptXLarge64 : kKptXLarge32;
    const int tv = tile_variant(n, wide);
    if (g_digit_bits == 4) {
        if (tv == 1) return sort_passes<K, small, 4>(keys, values, n, n_dev, key_bits, L, scratch, s);
        if (tv == 2) return sort_passes<K, large, 4>(keys, values, n, n_dev, key_bits, L, scratch, s);
        return sort_passes<K, xlarge, 4>(keys, values, n, n_dev, key_bits, L, scratch, s);
    }
    if (tv == 1) return sort_passes<K, small, 8>(keys, values, n, n_dev, key_bits, L, scratch, s);
    if (tv == 2) return sort_passes<K, large, 8>(keys, values, n, n_dev, key_bits, L, scratch, s);
    return sort_passes<K, xlarge, 8>(keys, values, n, n_dev, key_bits, L, scratch, s);
}

// Failure-detection self-test: one pass of a two-tile 32-bit sort run by a
// single CTA that draws ticket 1, so its look-back waits on tile 0, which
// nothing publishes.  The wait gives up after kSpinLimit polls and latches
// kErrTimeout; the scatter that follows writes only in-bounds slots (its
// positions are checked against the count).  Synchronises the stream.
cudaError_t sort_selftest_timeout(cudaStream_t s) {
    constexpr int KPT = kKptSmall32;
    constexpr uint32_t TILE = kSortThreads * KPT, N = 2 * TILE;
    cudaError_t e = sort_prepare();
    if (e != cudaSuccess) return e;
    uint32_t* buf = nullptr;  // keys, values, keys out, values out, ticket, lookback, histogram
    const size_t words = 4 * (size_t)N + 1 + 3 * kRadix;
    if ((e = dev_malloc(reinterpret_cast<void**>(&buf), words * sizeof(uint32_t))) != cudaSuccess) return e;
    uint32_t* keys = buf;
    uint32_t* vals = keys + N;
    uint32_t* keys_out = vals + N;
    uint32_t* vals_out = keys_out + N;
    uint32_t* ticket = vals_out + N;
    uint32_t* lookback = ticket + 1;
    uint32_t* hist = lookback + 2 * kRadix;  // zero: the global digit bases of an unsorted pass
    const uint32_t one = 1;
    e = cudaMemsetAsync(buf, 0, words * sizeof(uint32_t), s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ticket, &one, sizeof(one), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        k_onesweep<uint32_t, KPT, 8><<<1, kSortThreads, onesweep_smem<uint32_t, KPT, 8>(), s>>>(
            keys, vals, keys_out, vals_out, N, nullptr, 0, 0xFFu, hist, lookback, ticket, 0, 0u);
        count_launch();
        e = cudaGetLastError();
    }
    cudaError_t e2 = cudaStreamSynchronize(s);
    cudaFree(buf);
    return e != cudaSuccess ? e : e2;
}

cudaError_t launch_sort_pairs(void* keys, uint32_t* values, uint32_t n, const uint32_t* n_dev, int key_bits,
                              void* scratch, size_t scratch_bytes, cudaStream_t s) {
    (void)scratch_bytes;
    if (n == 0) return cudaSuccess;
    unsigned char* sc = reinterpret_cast<unsigned char*>(scratch);
    if (key_bits <= 32) return sort_impl<uint32_t>(reinterpret_cast<uint32_t*>(keys), values, n, n_dev, key_bits, sc, s);
    return sort_impl<uint64_t>(reinterpret_cast<uint64_t*>(keys), values, n, n_dev, key_bits, sc, s);
}

}  // namespace wfpt
