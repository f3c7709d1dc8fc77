// Hand-written device-wide primitives: single-pass prefix scan with fused load / store
// functors (decoupled look-back, dynamic tile ids, bounded waits) and a stable LSD radix
// sort of (32-bit key, 32-bit value) pairs.  Problem sizes are read from device memory.
#pragma once
#include "psr_common.cuh"

namespace psr {

constexpr int kScanItems = 8;                    // default items per thread
constexpr int kScanTile = kBlock * kScanItems;   // 2048 elements per default tile
constexpr int kScanMinTile = kBlock;             // smallest tile (1 item per thread)

// Scratch of the scans: [0] tile counter, [1] blocks finished, [2] epoch, [3 + t] status
// of tile t.  A status word is value (bits 0-31) | aggregate flag (32) | inclusive flag
// (33) | epoch (34-63); only statuses of the running launch's epoch count, so nothing is
// cleared between launches: the last block of a launch resets the counters and advances
// the epoch (launches on one stream are ordered, so the next launch sees both).
struct ScanScratch {
    unsigned long long* words;
    int max_tiles;
    int batch = 1;   // clouds of the launch (host side: the grid's y extent)
    __device__ void rebase() { PSR_CLOUD(words); }   // to cloud blockIdx.y
};
constexpr int kScanHeader = 3;

// optional count written by the last tile: min(total, cap) (overflow flags kErrCapacity)
struct ScanCount {
    int* dst = nullptr;
    int cap = 0;
    __device__ void rebase() { PSR_CLOUD(dst); }   // to cloud blockIdx.y
};

// Store functors may define `void done(unsigned total) const`: the scan calls it once, after
// the last element (or at once for an empty scan), to chain counts into the next launch.
template <class S>
__device__ __forceinline__ auto scan_done(const S& s, unsigned tot, int) -> decltype(s.done(tot), void()) {
    s.done(tot);
}
template <class S>
__device__ __forceinline__ void scan_done(const S&, unsigned, long) {}

constexpr unsigned long long kFlagAgg = 1ull << 32;
constexpr unsigned long long kFlagIncl = 1ull << 33;
constexpr int kEpochShift = 34;

__device__ __forceinline__ unsigned long long load_status(const unsigned long long* p) {
    return *((volatile const unsigned long long*)p);
}

// Block-wide exclusive scan of one value per thread; returns the block total.
__device__ __forceinline__ unsigned block_exclusive_scan(unsigned v, unsigned& excl, unsigned* smem_warp) {
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    unsigned x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (unsigned)o) x += y;
    }
    if (lane == 31) smem_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned w = (lane < (kBlock / 32)) ? smem_warp[lane] : 0u;
        unsigned s = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= (unsigned)o) s += y;
        }
        if (lane < (kBlock / 32)) smem_warp[lane] = s - w;   // exclusive warp offsets
        if (lane == (kBlock / 32) - 1) smem_warp[kBlock / 32] = s;
    }
    __syncthreads();
    excl = smem_warp[warp] + x - v;
    unsigned total = smem_warp[kBlock / 32];
    __syncthreads();
    return total;
}

// Generic scan.  Load(i) -> unsigned value of element i; Store(i, prefix, value) gets the
// exclusive prefix of element i.  *total receives the sum of all n elements.  kItems
// elements per thread: 8 for light functors, 1 or 2 where Load / Store do enough work per
// element that more, smaller tiles (more blocks in flight) pay.
template <int kItems, class Load, class Store>
__global__ void __launch_bounds__(kBlock) k_scan(Load load, Store store, const int* count_ptr, int count_add,
                                                 ScanScratch sc, unsigned* total, unsigned* err, ScanCount cnt) {
    PSR_CLOUD(load, store, count_ptr, sc, total, err, cnt);
    constexpr int kTile = kBlock * kItems;
    __shared__ unsigned s_warp[kBlock / 32 + 1];
    __shared__ int s_tile;
    __shared__ unsigned s_prefix;
    const int n = *count_ptr + count_add;
    const int ntiles = (n + kTile - 1) / kTile;
    if (n <= 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            *total = 0u;
            if (cnt.dst) *cnt.dst = 0;
            scan_done(store, 0u, 0);
        }
        return;
    }
    if (ntiles > sc.max_tiles) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(err, kErrCapacity);
        return;
    }
    unsigned long long* st = sc.words + kScanHeader;
    const unsigned long long epoch = load_status(sc.words + 2);
    const unsigned long long etag = epoch << kEpochShift;
    while (true) {
        if (threadIdx.x == 0) s_tile = (int)atomicAdd(sc.words, 1ull);
        __syncthreads();
        const int t = s_tile;
        __syncthreads();
        if (t >= ntiles) break;
        const int base = t * kTile + threadIdx.x * kItems;
        unsigned v[kItems];
        unsigned sum = 0;
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            int i = base + k;
            v[k] = (i < n) ? load(i) : 0u;
            sum += v[k];
        }
        unsigned excl;
        const unsigned agg = block_exclusive_scan(sum, excl, s_warp);
        // look-back by warp 0
        if (threadIdx.x < 32) {
            const unsigned lane = lane_id();
            if (t == 0) {
                if (lane == 0) {
                    atomicExch(st, etag | kFlagIncl | (unsigned long long)agg);
                    s_prefix = 0u;
                }
            } else {
                if (lane == 0) atomicExch(st + t, etag | kFlagAgg | (unsigned long long)agg);
                unsigned run = 0;
                int pred = t - 1;
                bool timeout = false;
                while (true) {
                    int idx = pred - (int)lane;
                    unsigned long long s = kFlagIncl;   // "prefix 0" past the first tile
                    if (idx >= 0) {
                        int it = 0;
                        s = load_status(st + idx);
                        while ((s >> kEpochShift) != epoch || !(s & (kFlagAgg | kFlagIncl))) {
                            if (++it > kSpinLimit) { timeout = true; s = kFlagIncl; break; }
                            __nanosleep(20);
                            s = load_status(st + idx);
                        }
                    }
                    unsigned incl_mask = __ballot_sync(0xffffffffu, (s & kFlagIncl) != 0);
                    unsigned val = (unsigned)(s & 0xffffffffull);
                    if (incl_mask) {
                        int first = __ffs(incl_mask) - 1;
                        unsigned contrib = ((int)lane <= first) ? val : 0u;
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1) contrib += __shfl_xor_sync(0xffffffffu, contrib, o);
                        run += contrib;
                        break;
                    }
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) val += __shfl_xor_sync(0xffffffffu, val, o);
                    run += val;
                    pred -= 32;
                }
                if (__any_sync(0xffffffffu, timeout) && lane == 0) atomicOr(err, kErrSpinTimeout);
                if (lane == 0) {
                    atomicExch(st + t, etag | kFlagIncl | (unsigned long long)(run + agg));
                    s_prefix = run;
                }
            }
        }
        __syncthreads();
        unsigned pre = s_prefix + excl;
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            int i = base + k;
            if (i < n) store(i, pre, v[k]);
            pre += v[k];
        }
        if (t == ntiles - 1 && threadIdx.x == kBlock - 1) {
            const unsigned tot = s_prefix + agg;
            *total = tot;
            if (cnt.dst) {
                int c = (int)tot;
                if (tot > (unsigned)cnt.cap) { atomicOr(err, kErrCapacity); c = cnt.cap; }
                *cnt.dst = c;
            }
            scan_done(store, tot, 0);
        }
        __syncthreads();
    }
    // every block ends here after claiming a tile past the end, i.e. after its last tile;
    // the last one to arrive resets the counters for the next launch
    if (threadIdx.x == 0) {
        const unsigned long long done = atomicAdd(sc.words + 1, 1ull);
        if (done == (unsigned long long)gridDim.x - 1) {
            atomicExch(sc.words, 0ull);
            atomicExch(sc.words + 1, 0ull);
            atomicExch(sc.words + 2, (epoch + 1) & ((1ull << (64 - kEpochShift)) - 1));
        }
    }
}

// blocks of a scan launch: blocks_per_sm per SM, at most max_tiles
int scan_grid(int max_tiles, int blocks_per_sm = 4);

// blocks_per_sm: 4 for scans that can be long (hundreds of tiles or more); small scans
// (per octree level, per point at a few hundred tiles) take 1 so that idle blocks do not
// occupy the GPU while other reconstructions run beside them
template <int kItems = kScanItems, class Load, class Store>
inline cudaError_t launch_scan(Load load, Store store, const int* count_ptr, int count_add, ScanScratch sc,
                               unsigned* total, unsigned* err, cudaStream_t stream, ScanCount cnt = ScanCount{},
                               int blocks_per_sm = 4) {
    const dim3 grid(cloud_blocks(sc.batch, scan_grid(sc.max_tiles, blocks_per_sm)), sc.batch);
    k_scan<kItems, Load, Store><<<grid, kBlock, 0, stream>>>(load, store, count_ptr, count_add, sc, total, err, cnt);
    return cudaGetLastError();
}

// ---- common load / store functors ----------------------------------------------------
struct LoadArray {
    const unsigned* a;
    __device__ unsigned operator()(int i) const { return a[i]; }
    __device__ void rebase() { PSR_CLOUD(a); }   // to cloud blockIdx.y
};
struct StoreExclusive {
    unsigned* out;
    __device__ void operator()(int i, unsigned pre, unsigned) const { out[i] = pre; }
    __device__ void rebase() { PSR_CLOUD(out); }   // to cloud blockIdx.y
};
struct StoreInclusive {
    unsigned* out;
    __device__ void operator()(int i, unsigned pre, unsigned v) const { out[i] = pre + v; }
    __device__ void rebase() { PSR_CLOUD(out); }   // to cloud blockIdx.y
};

// ---- radix sort ------------------------------------------------------------------------
constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kSortItems = 8;
constexpr int kSortTile = kBlock * kSortItems;   // 2048 keys per tile

struct SortScratch {
    unsigned* hist;          // [kRadix][max_tiles]
    unsigned* keys_alt;
    unsigned* vals_alt;
    int max_tiles;
    ScanScratch scan;
};

// n 32-bit words at p set to v, in each of `clouds` clouds (a memset that multi-cloud
// launches can take: every cloud's copy of the buffer)
cudaError_t fill_words(unsigned* p, unsigned v, long long n, int clouds, cudaStream_t stream);

cudaError_t radix_sort_pairs(unsigned* keys, unsigned* vals, const int* count_ptr, int key_bits, SortScratch sc,
                             unsigned* err, cudaStream_t stream, bool* result_in_alt);

}  // namespace psr
