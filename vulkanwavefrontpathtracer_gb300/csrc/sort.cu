// Stable LSD key/value radix sort, 8-bit digits, one sweep per digit.
//
// Replaces the reference's vrdxCmdSortKeyValue (upsweep -> spine ->
// downsweep per pass, external/vulkan_radix_sort/vk_radix_sort.h:2598-2755)
// with the single-sweep scheme of Adinets & Merrill ("Onesweep", 2022):
//   1. one histogram kernel reads the keys once and builds the 256-bin digit
//      histogram of every pass;
//   2. per pass, one kernel: each 256-thread CTA takes the next tile from a
//      ticket counter, ranks its keys with warp ballots (stable: keys are
//      ranked in input order), publishes its per-digit counts, resolves the
//      global digit offsets with a bounded decoupled look-back over earlier
//      tiles, stages the tile in shared memory in digit order and writes
//      keys and values out in coalesced runs.
// Ping-pong between the caller's buffers and scratch; after an even number
// of passes the result is back in the caller's buffers (as in the reference),
// after an odd number it is copied back.
#include <algorithm>
#include <utility>

#include "common.cuh"
#include "stages.cuh"

namespace wfpt {

cudaError_t status_sort(uint32_t* out) { return read_and_clear_status(out); }

constexpr int kSortBlock = 256;  // one thread per digit value
constexpr int kRadix = 256;
constexpr int kSortWarps = kSortBlock / 32;
constexpr uint32_t kLbAggregate = 1u << 30;
constexpr uint32_t kLbPrefix = 2u << 30;
constexpr uint32_t kLbValue = (1u << 30) - 1u;

template <typename K>
struct SortCfg;
template <>
struct SortCfg<uint32_t> {
    static constexpr int kKpt = 16;
};
template <>
struct SortCfg<uint64_t> {
    static constexpr int kKpt = 12;
};

template <typename K>
constexpr int tile_of() {
    return kSortBlock * SortCfg<K>::kKpt;
}

// Digit mask of pass p: the top pass keeps only the bits below key_bits.
__host__ __device__ __forceinline__ uint32_t pass_mask(int key_bits, int p) {
    int bits = key_bits - 8 * p;
    return bits >= 8 ? 0xFFu : ((1u << bits) - 1u);
}
__device__ __forceinline__ uint32_t digit_of(uint32_t k, int shift, uint32_t dmask) { return (k >> shift) & dmask; }
__device__ __forceinline__ uint32_t digit_of(uint64_t k, int shift, uint32_t dmask) { return (uint32_t)(k >> shift) & dmask; }

// Exclusive scan of one value per thread over a 256-thread block.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* s_warp) {
    uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    uint32_t off = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w)
        if (w < (int)warp) off += s_warp[w];
    __syncthreads();
    return off + x - v;
}

// Histogram of every pass's digit over the first `count` keys.
template <typename K>
__global__ void __launch_bounds__(kSortBlock) k_sort_hist(const K* __restrict__ keys, uint32_t n,
                                                           const uint32_t* __restrict__ n_dev, int passes,
                                                           int key_bits, uint32_t* __restrict__ hist) {
    __shared__ uint32_t s_h[8 * kRadix];
    for (int i = threadIdx.x; i < passes * kRadix; i += kSortBlock) s_h[i] = 0;
    __syncthreads();
    uint32_t count = load_count(n, n_dev);
    for (uint32_t i = blockIdx.x * kSortBlock + threadIdx.x; i < count; i += gridDim.x * kSortBlock) {
        K k = keys[i];
        for (int p = 0; p < passes; ++p) atomicAdd(&s_h[p * kRadix + digit_of(k, 8 * p, pass_mask(key_bits, p))], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * kRadix; i += kSortBlock) {
        uint32_t c = s_h[i];
        if (c) atomicAdd(&hist[i], c);
    }
}

// One digit pass.  Dynamic shared memory: TILE keys, TILE values,
// kSortWarps*256 per-warp digit counters, 256 global bases, 256 local offsets.
template <typename K>
__global__ void __launch_bounds__(kSortBlock, 4) k_onesweep(const K* __restrict__ keys_in,
                                                          const uint32_t* __restrict__ vals_in,
                                                          K* __restrict__ keys_out, uint32_t* __restrict__ vals_out,
                                                          uint32_t n, const uint32_t* __restrict__ n_dev, int shift, uint32_t dmask,
                                                          const uint32_t* __restrict__ hist,
                                                          uint32_t* __restrict__ lookback,
                                                          uint32_t* __restrict__ ticket) {
    constexpr int KPT = SortCfg<K>::kKpt;
    constexpr int TILE = kSortBlock * KPT;
    extern __shared__ __align__(16) unsigned char smem[];
    K* s_keys = reinterpret_cast<K*>(smem);
    uint32_t* s_vals = reinterpret_cast<uint32_t*>(s_keys + TILE);
    uint32_t* s_hist = s_vals + TILE;  // [warp][digit]
    uint32_t* s_base = s_hist + kSortWarps * kRadix;
    uint32_t* s_loc = s_base + kRadix;
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_scan[kSortWarps];

    const uint32_t count = load_count(n, n_dev);
    const uint32_t ntiles = (count + TILE - 1) / TILE;
    if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
    for (int i = threadIdx.x; i < kSortWarps * kRadix; i += kSortBlock) s_hist[i] = 0;
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile >= ntiles) return;

    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lt_mask = (1u << lane) - 1u;
    const uint32_t base = tile * TILE + warp * 32 * KPT + lane;

    K key[KPT];
    uint32_t rank[KPT];
#pragma unroll
    for (int k = 0; k < KPT; ++k) {
        uint32_t i = base + k * 32;
        key[k] = i < count ? keys_in[i] : (K)0;
    }
    uint32_t* my_hist = s_hist + warp * kRadix;
    // Warp-level stable ranking: keys are visited in input order (k, lane).
#pragma unroll
    for (int k = 0; k < KPT; ++k) {
        bool ok = (base + k * 32) < count;
        uint32_t d = digit_of(key[k], shift, dmask);
        uint32_t peers = __ballot_sync(0xffffffffu, ok);
#pragma unroll
        for (int b = 0; b < 8; ++b) {
            uint32_t bit = (d >> b) & 1u;
            uint32_t m = __ballot_sync(0xffffffffu, bit);
            peers &= bit ? m : ~m;
        }
        uint32_t before = peers & lt_mask;
        uint32_t pre = ok ? my_hist[d] : 0u;
        __syncwarp();
        if (ok && before == 0u) my_hist[d] = pre + __popc(peers);
        __syncwarp();
        rank[k] = pre + __popc(before);
    }
    __syncthreads();

    // Thread t owns digit t: warp-exclusive prefixes and the tile count.
    const uint32_t d = threadIdx.x;
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) {
        uint32_t c = s_hist[w * kRadix + d];
        s_hist[w * kRadix + d] = run;
        run += c;
    }
    // Decoupled look-back for digit d.
    uint32_t* lb = lookback + (size_t)tile * kRadix + d;
    uint32_t excl;
    if (tile == 0) {
        // Global exclusive digit offset from the histogram.
        excl = block_exclusive_scan(hist[d], s_scan);
        atomicExch(lb, kLbPrefix | (excl + run));
    } else {
        atomicExch(lb, kLbAggregate | run);
        excl = 0;
        // Walk back over predecessors, reading kChunk of them with
        // independent loads per round trip; stop at the first inclusive
        // prefix, wait (bounded) on an entry that is not published yet.
        constexpr int kChunk = 8;
        int32_t j = (int32_t)tile - 1;
        uint32_t spins = 0;
        bool done = false;
        while (!done && j >= 0) {
            uint32_t st[kChunk];
#pragma unroll
            for (int q = 0; q < kChunk; ++q)
                st[q] = (j - q >= 0) ? *((volatile uint32_t*)(lookback + (size_t)(j - q) * kRadix + d))
                                     : uint32_t(kLbPrefix);
            int used = 0;
#pragma unroll
            for (int q = 0; q < kChunk; ++q) {
                if (done || used < q) continue;  // stopped earlier in this chunk
                uint32_t flag = st[q] & ~kLbValue;
                if (flag == 0u) continue;  // not published: re-read from here
                excl += st[q] & kLbValue;
                used = q + 1;
                if (flag == kLbPrefix) done = true;
            }
            j -= used;
            if (!done && used < kChunk && j >= 0) {
                if (++spins > kSpinLimit) {
                    raise_status(kErrTimeout);
                    break;
                }
                __nanosleep(32);
            }
        }
        atomicExch(lb, kLbPrefix | (excl + run));
    }
    uint32_t loc = block_exclusive_scan(run, s_scan);
    s_loc[d] = loc;
    s_base[d] = excl - loc;
    __syncthreads();

    // Stage the tile in digit order; values are read here, straight from
    // global memory into their sorted slot.
#pragma unroll
    for (int k = 0; k < KPT; ++k) {
        uint32_t i = base + k * 32;
        if (i < count) {
            uint32_t dk = digit_of(key[k], shift, dmask);
            uint32_t pos = s_loc[dk] + my_hist[dk] + rank[k];
            s_keys[pos] = key[k];
            s_vals[pos] = vals_in[i];
        }
    }
    __syncthreads();
    const uint32_t tile_count = min((uint32_t)TILE, count - tile * TILE);
    for (uint32_t j = threadIdx.x; j < tile_count; j += kSortBlock) {
        K kk = s_keys[j];
        uint32_t g = s_base[digit_of(kk, shift, dmask)] + j;
        if (g < count) {  // only fails after a look-back timeout
            keys_out[g] = kk;
            vals_out[g] = s_vals[j];
        } else {
            raise_status(kErrBounds);
        }
    }
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

template <typename K>
static size_t onesweep_smem() {
    constexpr int TILE = tile_of<K>();
    return (size_t)TILE * sizeof(K) + (size_t)TILE * 4 + (size_t)(kSortWarps + 2) * kRadix * 4;
}

// Opts the pass kernels into their dynamic shared memory once (not a stream
// operation, so the renderer calls it before capturing a frame graph).
cudaError_t sort_prepare() {
    static bool done = false;
    if (done) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(k_onesweep<uint32_t>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)onesweep_smem<uint32_t>());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_onesweep<uint64_t>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)onesweep_smem<uint64_t>());
    if (e == cudaSuccess) done = true;
    return e;
}

struct SortLayout {
    int passes;
    size_t key_bytes;
    size_t tiles;
    size_t off_ticket, off_hist, off_lookback, off_keys, off_vals, total;
};

static SortLayout sort_layout(uint32_t max_n, int key_bits) {
    SortLayout L;
    L.passes = (key_bits + 7) / 8;
    L.key_bytes = key_bits <= 32 ? 4 : 8;
    size_t tile = key_bits <= 32 ? tile_of<uint32_t>() : tile_of<uint64_t>();
    L.tiles = ((size_t)max_n + tile - 1) / tile;
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

template <typename K>
static cudaError_t sort_impl(K* keys, uint32_t* values, uint32_t n, const uint32_t* n_dev, int key_bits,
                             unsigned char* scratch, cudaStream_t s) {
    SortLayout L = sort_layout(n, key_bits);
    // Tickets, histograms and look-back states start at zero.
    cudaError_t e = cudaMemsetAsync(scratch, 0, L.off_keys, s);
    if (e != cudaSuccess) return e;
    uint32_t* tickets = reinterpret_cast<uint32_t*>(scratch + L.off_ticket);
    uint32_t* hist = reinterpret_cast<uint32_t*>(scratch + L.off_hist);
    uint32_t* lookback = reinterpret_cast<uint32_t*>(scratch + L.off_lookback);
    K* alt_keys = reinterpret_cast<K*>(scratch + L.off_keys);
    uint32_t* alt_vals = reinterpret_cast<uint32_t*>(scratch + L.off_vals);

    unsigned hgrid = (unsigned)std::min<size_t>(((size_t)n + kSortBlock * 8 - 1) / (kSortBlock * 8), 152 * 4);
    if (hgrid == 0) hgrid = 1;
    k_sort_hist<K><<<hgrid, kSortBlock, 0, s>>>(keys, n, n_dev, L.passes, key_bits, hist);
    count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;

    size_t smem = onesweep_smem<K>();
    if ((e = sort_prepare()) != cudaSuccess) return e;
    K* src_k = keys;
    uint32_t* src_v = values;
    K* dst_k = alt_keys;
    uint32_t* dst_v = alt_vals;
    unsigned grid = (unsigned)(L.tiles == 0 ? 1 : L.tiles);
    for (int p = 0; p < L.passes; ++p) {
        k_onesweep<K><<<grid, kSortBlock, smem, s>>>(src_k, src_v, dst_k, dst_v, n, n_dev, 8 * p, pass_mask(key_bits, p),
                                                     hist + p * kRadix, lookback + (size_t)p * L.tiles * kRadix,
                                                     tickets + p);
        count_launch();
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        std::swap(src_k, dst_k);
        std::swap(src_v, dst_v);
    }
    if (L.passes & 1) {
        unsigned cgrid = (unsigned)std::min<size_t>(((size_t)n + kSortBlock - 1) / kSortBlock, 152 * 16);
        k_copy_back<K><<<cgrid, kSortBlock, 0, s>>>(alt_keys, alt_vals, keys, values, n, n_dev);
        count_launch();
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
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
