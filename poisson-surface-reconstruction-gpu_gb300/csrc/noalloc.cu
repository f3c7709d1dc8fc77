// Morton encoding + stable radix sort of a point cloud without any device allocation.
//
// Some callers cannot call cudaMalloc at all: code running under a caller-owned memory
// pool or arena that forbids outside allocations, plug-ins loaded into a host process
// whose allocator must see every byte, and real-time loops where an allocation (and the
// implicit synchronisation it can cause) is not allowed.  For them this file provides
// psr_morton_sort_noalloc, the point-ordering step of the pipeline (bounding box,
// normalisation, Morton code, stable sort by code) with all of its scratch in a
// file-scope __device__ array of fixed size.  The caller passes the input points and the
// two output arrays; the call allocates nothing.
//
// Limits and sharing:
//   * at most kNoAllocMaxPoints points per call (larger calls are rejected with
//     PSR_OUT_OF_CAPACITY);
//   * the scratch array lives on every device that loads this library, for the life of
//     the process, and is shared by all calls on that device: it keeps the last call's
//     contents (everything that must start at zero is cleared by each call), and calls
//     whose GPU work overlaps in time race on it;
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) with that device current;
//   * every call waits for its own work on `stream` (it reads the device error word back
//     and synchronises that stream), so it must not be called while any stream of the
//     device is being captured into a CUDA graph.
#include <mutex>

#include "../../include/psr/psr.h"
#include "primitives.cuh"

namespace psr {

constexpr int kNoAllocMaxPoints = 1 << 20;
constexpr int kNoAllocSortTiles = (kNoAllocMaxPoints + kSortTile - 1) / kSortTile + 1;
constexpr int kNoAllocScanTiles = (kRadix * kNoAllocSortTiles + kScanTile - 1) / kScanTile + 2;

struct NoAllocState {
    int n;
    unsigned error;
    int bmax[3], bmin[3];
    float center[3];
    float edge;
};

// scratch layout (all offsets 256-byte aligned)
constexpr size_t kNaState = 0;
constexpr size_t kNaKeys = 256;
constexpr size_t kNaVals = kNaKeys + 4ull * kNoAllocMaxPoints;
constexpr size_t kNaHist = kNaVals + 4ull * kNoAllocMaxPoints;
constexpr size_t kNaHistBytes = ((4ull * ((size_t)kRadix * kNoAllocSortTiles + 16)) + 255) & ~255ull;
constexpr size_t kNaScan = kNaHist + kNaHistBytes;
constexpr size_t kNaBytes = kNaScan + 8ull * (kNoAllocScanTiles + kScanHeader);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

__global__ void k_na_init(NoAllocState* st, int n) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        st->n = n;
        st->error = 0;
        for (int a = 0; a < 3; ++a) {
            // seeded like the pipeline's reduction (-FLT_MAX / FLT_MAX), so the two agree
            // for coordinates of any magnitude
            st->bmax[a] = float_to_ordered(-FLT_MAX);
            st->bmin[a] = float_to_ordered(FLT_MAX);
        }
    }
}

__global__ void __launch_bounds__(kBlock) k_na_bbox(const float* xyz, NoAllocState* st) {
    const int n = st->n;
    float mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX}, mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
    bool bad = false;
    PSR_GRID_STRIDE(i, n) {
        for (int a = 0; a < 3; ++a) {
            const float v = xyz[3 * (size_t)i + a];
            if (!isfinite(v)) bad = true;
            mx[a] = mx[a] < v ? v : mx[a];
            mn[a] = mn[a] > v ? v : mn[a];
        }
    }
    for (int a = 0; a < 3; ++a)
        for (int o = 16; o > 0; o >>= 1) {
            mx[a] = fmaxf(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
            mn[a] = fminf(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
        }
    if (__any_sync(0xffffffffu, bad) && lane_id() == 0) atomicOr(&st->error, kErrInvalid);
    if (lane_id() == 0)
        for (int a = 0; a < 3; ++a) {
            atomicMax(&st->bmax[a], float_to_ordered(mx[a]));
            atomicMin(&st->bmin[a], float_to_ordered(mn[a]));
        }
}

// same arithmetic as the pipeline's bounding-box step (mesh/BuildOctree.cu:619-631)
__global__ void k_na_finalize(NoAllocState* st, float scale) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    float edge = 1.0f, ctr[3];
    for (int a = 0; a < 3; ++a) {
        const float mx = ordered_to_float(st->bmax[a]), mn = ordered_to_float(st->bmin[a]);
        const float ext = __fsub_rn(mx, mn);
        if (a == 0 || edge < ext) edge = ext;
        ctr[a] = __fdiv_rn(__fadd_rn(mx, mn), 2.0f);
    }
    edge = __fmul_rn(edge, __fmul_rn(scale, 1.0f));
    for (int a = 0; a < 3; ++a) st->center[a] = __fsub_rn(ctr[a], __fdiv_rn(edge, 2.0f));
    st->edge = edge;
    if (!(edge > 0.0f)) atomicOr(&st->error, kErrInvalid);
}

__global__ void __launch_bounds__(kBlock) k_na_encode(const float* xyz, const NoAllocState* st, int depth,
                                                      unsigned* code, unsigned* order) {
    const int n = st->n;
    const float e = st->edge;
    PSR_GRID_STRIDE(i, n) {
        float p[3];
        for (int a = 0; a < 3; ++a)
            p[a] = __fdiv_rn(__fmul_rn(__fsub_rn(xyz[3 * (size_t)i + a], st->center[a]), 1.0f), e);
        unsigned k = 0;
        float cc[3] = {0.5f, 0.5f, 0.5f};
        float w = 0.25f;
        for (int l = depth - 1; l >= 0; --l) {
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                if (p[a] > cc[a]) { k |= 1u << (3 * l + 2 - a); cc[a] = __fadd_rn(cc[a], w); }
                else cc[a] = __fsub_rn(cc[a], w);
            }
            w = __fdiv_rn(w, 2.0f);
        }
        code[i] = k;
        order[i] = (unsigned)i;
    }
}

namespace {
std::mutex g_na_mutex;
unsigned char* g_na_ptr[64] = {};   // device address of the scratch array, per device ordinal
}  // namespace

}  // namespace psr

using namespace psr;

// psr_morton_sort_noalloc: see include/psr/psr.h.  Returns after the work on `stream` has
// completed (it reads back the device error word).
extern "C" psr_status psr_morton_sort_noalloc(const float* xyz, int count, int depth, float bbox_scale,
                                              uint32_t* codes, uint32_t* order, void* stream) {
    if (!xyz || !codes || !order || count <= 0 || depth < 1 || depth > kMaxDepth || !(bbox_scale > 0.0f))
        return PSR_INVALID_INPUT;
    if (count > kNoAllocMaxPoints) return PSR_OUT_OF_CAPACITY;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return PSR_CUDA_ERROR;
    unsigned char* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_na_mutex);
        if (!g_na_ptr[dev]) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) return PSR_CUDA_ERROR;
            g_na_ptr[dev] = (unsigned char*)p;
        }
        base = g_na_ptr[dev];
    }
    cudaStream_t s = (cudaStream_t)stream;
    NoAllocState* st = (NoAllocState*)(base + kNaState);
    SortScratch sc;
    sc.hist = (unsigned*)(base + kNaHist);
    sc.keys_alt = (unsigned*)(base + kNaKeys);
    sc.vals_alt = (unsigned*)(base + kNaVals);
    sc.max_tiles = kNoAllocSortTiles;
    sc.scan.words = (unsigned long long*)(base + kNaScan);
    sc.scan.max_tiles = kNoAllocScanTiles;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = (sms > 0 ? sms : 148) * 4;
    k_na_init<<<1, 1, 0, s>>>(st, count);
    k_na_bbox<<<grid, kBlock, 0, s>>>(xyz, st);
    k_na_finalize<<<1, 1, 0, s>>>(st, bbox_scale);
    k_na_encode<<<grid, kBlock, 0, s>>>(xyz, st, depth, codes, order);
    bool alt = false;
    cudaError_t e = radix_sort_pairs(codes, order, &st->n, 3 * depth, sc, &st->error, s, &alt);
    if (e == cudaSuccess && alt) {
        e = cudaMemcpyAsync(codes, sc.keys_alt, 4 * (size_t)count, cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(order, sc.vals_alt, 4 * (size_t)count, cudaMemcpyDeviceToDevice, s);
    }
    // the error word is read on the caller's stream only: no other stream of the device
    // is waited on
    unsigned err = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&err, &st->error, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return PSR_CUDA_ERROR;
    if (err & kErrInvalid) return PSR_INVALID_INPUT;
    if (err & kErrCapacity) return PSR_OUT_OF_CAPACITY;
    if (err & kErrSpinTimeout) return PSR_DEVICE_TIMEOUT;
    return PSR_OK;
}
