// Hand-written radix sort (stable LSD, 8-bit digits) built on the look-back scan.
#include "primitives.cuh"

namespace psr {

static int g_num_sms = 0;

int scan_grid(int max_tiles, int blocks_per_sm) {
    if (g_num_sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_num_sms <= 0) g_num_sms = 148;
    }
    int g = g_num_sms * blocks_per_sm;
    return g < max_tiles ? g : (max_tiles > 0 ? max_tiles : 1);
}

// Per-tile digit histogram, digit-major layout hist[digit * max_tiles + tile].
__global__ void __launch_bounds__(kBlock) k_sort_hist(const unsigned* keys, const int* count_ptr, int shift,
                                                      unsigned* hist, int max_tiles, unsigned* err) {
    PSR_CLOUD(keys, count_ptr, hist, err);
    __shared__ unsigned s_h[kRadix];
    const int n = *count_ptr;
    const int ntiles = (n + kSortTile - 1) / kSortTile;
    if (ntiles > max_tiles) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(err, kErrCapacity);
        return;
    }
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        for (int d = threadIdx.x; d < kRadix; d += kBlock) s_h[d] = 0;
        __syncthreads();
        const int base = t * kSortTile;
        for (int k = threadIdx.x; k < kSortTile; k += kBlock) {
            int i = base + k;
            if (i < n) atomicAdd(&s_h[(keys[i] >> shift) & (kRadix - 1)], 1u);
        }
        __syncthreads();
        for (int d = threadIdx.x; d < kRadix; d += kBlock) hist[(size_t)d * max_tiles + t] = s_h[d];
        __syncthreads();
    }
}

struct HistLoad {
    const unsigned* hist;
    const int* count_ptr;
    int max_tiles;
    __device__ unsigned operator()(int i) const {
        int nt = (*count_ptr + kSortTile - 1) / kSortTile;
        int d = i / nt, t = i - d * nt;
        return hist[(size_t)d * max_tiles + t];
    }
    __device__ void rebase() { PSR_CLOUD(hist, count_ptr); }   // to cloud blockIdx.y
};
struct HistStore {
    unsigned* hist;
    const int* count_ptr;
    int max_tiles;
    __device__ void operator()(int i, unsigned pre, unsigned) const {
        int nt = (*count_ptr + kSortTile - 1) / kSortTile;
        int d = i / nt, t = i - d * nt;
        hist[(size_t)d * max_tiles + t] = pre;
    }
    __device__ void rebase() { PSR_CLOUD(hist, count_ptr); }   // to cloud blockIdx.y
};

// number of histogram entries to scan = kRadix * ntiles, written to *n_out
__global__ void k_sort_hist_count(const int* count_ptr, int* n_out) {
    PSR_CLOUD(count_ptr, n_out);
    int n = *count_ptr;
    *n_out = kRadix * ((n + kSortTile - 1) / kSortTile);
}

// Stable scatter.  Within a tile, warp w owns keys [w*256, w*256+256) in striped order
// (item j of lane l is key w*256 + 32*j + l), so processing items in order and ranking
// equal digits with __match_any_sync preserves the input order.
__global__ void __launch_bounds__(kBlock) k_sort_scatter(const unsigned* keys_in, const unsigned* vals_in,
                                                         unsigned* keys_out, unsigned* vals_out,
                                                         const int* count_ptr, int shift, const unsigned* offs,
                                                         int max_tiles) {
    PSR_CLOUD(keys_in, vals_in, keys_out, vals_out, count_ptr, offs);
    __shared__ unsigned s_cnt[kBlock / 32][kRadix];
    const int n = *count_ptr;
    const int ntiles = (n + kSortTile - 1) / kSortTile;
    if (ntiles > max_tiles) return;
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        for (int d = threadIdx.x; d < kRadix * (kBlock / 32); d += kBlock) (&s_cnt[0][0])[d] = 0;
        __syncthreads();
        const int base = t * kSortTile + warp * 256;
        unsigned key[kSortItems], val[kSortItems], rank[kSortItems];
        bool ok[kSortItems];
#pragma unroll
        for (int j = 0; j < kSortItems; ++j) {
            int i = base + 32 * j + lane;
            ok[j] = i < n;
            key[j] = ok[j] ? keys_in[i] : 0u;
            val[j] = ok[j] ? vals_in[i] : 0u;
            unsigned dgt = (key[j] >> shift) & (kRadix - 1);
            unsigned act = __ballot_sync(0xffffffffu, ok[j]);
            rank[j] = 0;
            if (ok[j]) {
                unsigned peers = __match_any_sync(act, dgt);
                unsigned before = __popc(peers & lt_mask);
                unsigned cur = s_cnt[warp][dgt];
                rank[j] = cur + before;
                __syncwarp(act);
                if (before == 0) s_cnt[warp][dgt] = cur + __popc(peers);
            }
            __syncwarp();
        }
        __syncthreads();
        // per-digit exclusive prefix over warps (in place)
        for (int d = threadIdx.x; d < kRadix; d += kBlock) {
            unsigned run = 0;
#pragma unroll
            for (int w = 0; w < kBlock / 32; ++w) {
                unsigned c = s_cnt[w][d];
                s_cnt[w][d] = run;
                run += c;
            }
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < kSortItems; ++j) {
            if (!ok[j]) continue;
            unsigned dgt = (key[j] >> shift) & (kRadix - 1);
            unsigned pos = offs[(size_t)dgt * max_tiles + t] + s_cnt[warp][dgt] + rank[j];
            keys_out[pos] = key[j];
            vals_out[pos] = val[j];
        }
        __syncthreads();
    }
}

// p[0 .. n) = v, in every cloud of the launch
__global__ void __launch_bounds__(kBlock) k_fill_words(unsigned* p, unsigned v, long long n) {
    PSR_CLOUD(p);
    for (long long i = blockIdx.x * (long long)kBlock + threadIdx.x; i < n; i += (long long)gridDim.x * kBlock) p[i] = v;
}

cudaError_t fill_words(unsigned* p, unsigned v, long long n, int clouds, cudaStream_t stream) {
    const long long g = (n + kBlock - 1) / kBlock;
    const int cap = scan_grid(1 << 30, 4);
    const int gx = (int)(g < cap ? (g < 1 ? 1 : g) : cap);
    k_fill_words<<<dim3(cloud_blocks(clouds, gx), clouds), kBlock, 0, stream>>>(p, v, n);
    return cudaGetLastError();
}

cudaError_t radix_sort_pairs(unsigned* keys, unsigned* vals, const int* count_ptr, int key_bits, SortScratch sc,
                             unsigned* err, cudaStream_t stream, bool* result_in_alt) {
    int passes = (key_bits + kRadixBits - 1) / kRadixBits;
    if (passes < 1) passes = 1;
    unsigned *ki = keys, *vi = vals, *ko = sc.keys_alt, *vo = sc.vals_alt;
    const int nb = sc.scan.batch;
    const dim3 grid(cloud_blocks(nb, scan_grid(sc.max_tiles)), nb);
    // the histogram scan length lives in the last int of the hist scratch area
    int* n_hist = (int*)(sc.hist + (size_t)kRadix * sc.max_tiles);
    unsigned* total = (unsigned*)(n_hist + 1);
    for (int p = 0; p < passes; ++p) {
        const int shift = p * kRadixBits;
        k_sort_hist<<<grid, kBlock, 0, stream>>>(ki, count_ptr, shift, sc.hist, sc.max_tiles, err);
        k_sort_hist_count<<<dim3(1, nb), 1, 0, stream>>>(count_ptr, n_hist);
        cudaError_t e = launch_scan(HistLoad{sc.hist, count_ptr, sc.max_tiles}, HistStore{sc.hist, count_ptr, sc.max_tiles},
                                    n_hist, 0, sc.scan, total, err, stream, ScanCount{}, 1);
        if (e != cudaSuccess) return e;
        k_sort_scatter<<<grid, kBlock, 0, stream>>>(ki, vi, ko, vo, count_ptr, shift, sc.hist, sc.max_tiles);
        unsigned* tk = ki; ki = ko; ko = tk;
        unsigned* tv = vi; vi = vo; vo = tv;
    }
    *result_in_alt = (passes & 1) != 0;
    return cudaGetLastError();
}

}  // namespace psr
