// Handle, workspace allocation and the C ABI (include/psr/psr.h).
#include <cuda.h>
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "../../include/psr/psr.h"
#include "workspace.h"

namespace psr {
cudaError_t upload_tables_octree();
cudaError_t upload_tables_field();
cudaError_t upload_tables_solver();
cudaError_t upload_tables_mesh();
cudaError_t upload_tables_transfer();
cudaError_t normals_build(Workspace& ws, const float* xyz, int n, float* out, float vpx, float vpy, float vpz);
cudaError_t weld_build(Workspace& ws);
void build_dff_table(int depth, std::vector<double>& dff);
void build_stencil(int depth, std::vector<float>& st, double eps);
}  // namespace psr

using namespace psr;

// CG iterations between true-residual evaluations (psr_config.cg_residual_period = 0)
constexpr int kDefaultResidualPeriod = 32;

struct DebugArray {
    const void* ptr;
    int elem;        // bytes per element
    int kind;        // 0 int32, 1 float32, 2 float64, 3 uint8, 4 uint16
    const int* count_field;   // device counter (nullptr: fixed count)
    long long fixed;
    int mult;        // elements per counted item
};

struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    int kernels = 0;
};

struct psr_handle {
    psr_config cfg;
    Workspace ws;
    int* h_params = nullptr;   // pinned: written by the host, copied to ws.d_params per call
    std::map<long long, GraphEntry> graphs;
    int use_graphs = 1;
    int last_kernels = 0;
    int last_graph = 0;
    void* arena = nullptr;
    size_t arena_bytes = 0;
    cudaStream_t own_stream = nullptr;
    cudaEvent_t ev[7] = {};   // stage boundaries 0..5, end of the CG kernel 6
    Counters host_cnt;
    bool have_result = false;
    std::string last_error;
    psr_stats stats;
    // the reconstruction in flight (psr_submit / psr_submit_batch ... psr_poll / psr_wait)
    cudaEvent_t done = nullptr;
    bool pending = false;
    bool pend_batch = false;
    std::vector<psr_mesh> pend_meshes;        // copies of the callers' mesh descriptors
    std::vector<char> pend_emitted;           // per cloud: outputs written by the GPU
    psr_mesh* pend_user_mesh = nullptr;       // single call: the caller's descriptor
    psr_mesh* pend_user_meshes = nullptr;     // batch call: the callers' descriptors
    int pend_depth = 0, pend_colour = 0, pend_normals = 0;
    cudaStream_t pend_stream = nullptr;
    // cloud slots: 1, or batch_clouds workspaces mapped kCloudStride apart
    int clouds = 1;
    unsigned long long va_base = 0;           // reserved address range of a batch handle
    size_t va_slot = 0;                       // bytes mapped per slot
    Counters* cnt_host_all = nullptr;         // pinned count read-back, one per slot
    std::vector<psr_stats> batch_stats;       // per cloud of the last completed call
    std::vector<psr_status> batch_status;
};

namespace {

struct Arena {
    size_t bytes = 0;
    std::vector<std::pair<void**, size_t>> items;
    template <class T>
    void add(T*& p, size_t count) {
        items.push_back({(void**)&p, count * sizeof(T)});
        bytes += (count * sizeof(T) + 255) & ~(size_t)255;
    }
    void assign(char* base) {
        size_t off = 0;
        for (auto& it : items) {
            *it.first = base + off;
            off += (it.second + 255) & ~(size_t)255;
        }
    }
};

psr_status fail(psr_handle* h, psr_status s, const char* msg) {
    if (h) h->last_error = msg ? msg : "";
    return s;
}

psr_status cuda_fail(psr_handle* h, cudaError_t e, const char* where) {
    if (h) h->last_error = std::string(where) + ": " + cudaGetErrorString(e);
    return PSR_CUDA_ERROR;
}

// Cloud k's copy of a workspace buffer of a batch handle.
template <class T>
T* slot_ptr(T* p, int k) {
    return p ? (T*)((char*)p + (unsigned long long)k * kCloudStride) : p;
}

// ---- cloud slots of a batch handle ---------------------------------------------------
// One address range of batch_clouds * kCloudStride bytes, aligned to kMaxBatchClouds *
// kCloudStride, is reserved and every slot's workspace is backed by its own physical
// allocation mapped at the slot's start, so slot k's buffers sit exactly k * kCloudStride
// bytes after slot 0's (the kernels' PSR_CLOUD rebasing).  The driver's virtual-memory
// calls are reached through the runtime's driver entry points (no link-time dependency
// on the driver library).
typedef CUresult (*PfnGranularity)(size_t*, const CUmemAllocationProp*, CUmemAllocationGranularity_flags);
typedef CUresult (*PfnReserve)(CUdeviceptr*, size_t, size_t, CUdeviceptr, unsigned long long);
typedef CUresult (*PfnAddressFree)(CUdeviceptr, size_t);
typedef CUresult (*PfnCreate)(CUmemGenericAllocationHandle*, size_t, const CUmemAllocationProp*, unsigned long long);
typedef CUresult (*PfnRelease)(CUmemGenericAllocationHandle);
typedef CUresult (*PfnMap)(CUdeviceptr, size_t, size_t, CUmemGenericAllocationHandle, unsigned long long);
typedef CUresult (*PfnUnmap)(CUdeviceptr, size_t);
typedef CUresult (*PfnSetAccess)(CUdeviceptr, size_t, const CUmemAccessDesc*, size_t);

struct VmmApi {
    PfnGranularity granularity = nullptr;
    PfnReserve reserve = nullptr;
    PfnAddressFree address_free = nullptr;
    PfnCreate create = nullptr;
    PfnRelease release = nullptr;
    PfnMap map = nullptr;
    PfnUnmap unmap = nullptr;
    PfnSetAccess set_access = nullptr;
    bool ok = false;
};

const VmmApi& vmm() {
    static VmmApi api = [] {
        VmmApi a;
        auto get = [](const char* name, void** fn) {
            cudaDriverEntryPointQueryResult q;
            return cudaGetDriverEntryPointByVersion(name, fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
                   q == cudaDriverEntryPointSuccess && *fn;
        };
        a.ok = get("cuMemGetAllocationGranularity", (void**)&a.granularity) &&
               get("cuMemAddressReserve", (void**)&a.reserve) && get("cuMemAddressFree", (void**)&a.address_free) &&
               get("cuMemCreate", (void**)&a.create) && get("cuMemRelease", (void**)&a.release) &&
               get("cuMemMap", (void**)&a.map) && get("cuMemUnmap", (void**)&a.unmap) &&
               get("cuMemSetAccess", (void**)&a.set_access);
        return a;
    }();
    return api;
}

// Unmaps the first `mapped` slots and frees the reserved range.
void release_cloud_slots(psr_handle* h, int mapped) {
    const VmmApi& v = vmm();
    for (int k = 0; k < mapped; ++k) v.unmap((CUdeviceptr)(h->va_base + (unsigned long long)k * kCloudStride), h->va_slot);
    v.address_free((CUdeviceptr)h->va_base, (size_t)h->clouds * kCloudStride);
    h->va_base = 0;
    h->va_slot = 0;
}

psr_status map_cloud_slots(psr_handle* h, size_t bytes) {
    const VmmApi& v = vmm();
    if (!v.ok) return fail(h, PSR_CUDA_ERROR, "virtual memory management calls unavailable");
    CUmemAllocationProp prop = {};
    prop.type = CU_MEM_ALLOCATION_TYPE_PINNED;
    prop.location.type = CU_MEM_LOCATION_TYPE_DEVICE;
    prop.location.id = h->cfg.device;
    size_t gran = 0;
    if (v.granularity(&gran, &prop, CU_MEM_ALLOC_GRANULARITY_RECOMMENDED) != CUDA_SUCCESS || gran == 0)
        return fail(h, PSR_CUDA_ERROR, "cuMemGetAllocationGranularity");
    const size_t slot = (bytes + gran - 1) / gran * gran;
    if (slot > kCloudStride) return fail(h, PSR_OUT_OF_CAPACITY, "one cloud's workspace exceeds the slot stride");
    CUdeviceptr base = 0;
    if (v.reserve(&base, (size_t)h->clouds * kCloudStride, (size_t)kMaxBatchClouds * kCloudStride, 0, 0) !=
            CUDA_SUCCESS ||
        (((unsigned long long)base >> 35) & (kMaxBatchClouds - 1)) != 0)
        return fail(h, PSR_CUDA_ERROR, "cuMemAddressReserve");
    h->va_base = (unsigned long long)base;
    h->va_slot = slot;
    CUmemAccessDesc acc = {};
    acc.location = prop.location;
    acc.flags = CU_MEM_ACCESS_FLAGS_PROT_READWRITE;
    for (int k = 0; k < h->clouds; ++k) {
        const CUdeviceptr at = base + (CUdeviceptr)((unsigned long long)k * kCloudStride);
        CUmemGenericAllocationHandle mh;
        if (v.create(&mh, slot, &prop, 0) != CUDA_SUCCESS) {
            release_cloud_slots(h, k);
            return fail(h, PSR_OUT_OF_CAPACITY, "cuMemCreate: not enough device memory for the cloud slots");
        }
        const bool mapped = v.map(at, slot, 0, mh, 0) == CUDA_SUCCESS;
        v.release(mh);   // the mapping keeps the memory until it is unmapped
        if (!mapped || v.set_access(at, slot, &acc, 1) != CUDA_SUCCESS) {
            release_cloud_slots(h, k + (mapped ? 1 : 0));
            return fail(h, PSR_CUDA_ERROR, "cuMemMap / cuMemSetAccess");
        }
    }
    return PSR_OK;
}

}  // namespace

extern "C" {

psr_status psr_config_default(psr_config* c) {
    if (!c) return PSR_INVALID_INPUT;
    memset(c, 0, sizeof(*c));
    c->max_depth = 7;
    c->max_points = 300000;
    c->max_triangles = 1000000;
    c->max_mesh_vertices = 300000;
    c->max_nodes = 0;
    c->max_subdivision_nodes = 0;
    c->bbox_scale = 1.25f;
    c->cg_max_iterations = 10000;
    c->cg_tolerance = 1e-5f;
    c->laplacian_epsilon = 1e-6f;
    c->concurrent_stages = 1;
    c->compute_colors = 0;
    c->compute_normals = 0;
    c->weld_vertices = 0;
    c->device = 0;
    return PSR_OK;
}

const char* psr_status_string(psr_status s) {
    switch (s) {
        case PSR_OK: return "ok";
        case PSR_OUT_OF_CAPACITY: return "out of capacity";
        case PSR_INVALID_INPUT: return "invalid input";
        case PSR_NONCONVERGED: return "not converged";
        case PSR_DEVICE_TIMEOUT: return "device timeout";
        case PSR_CUDA_ERROR: return "cuda error";
        case PSR_PENDING: return "pending";
    }
    return "unknown";
}

const char* psr_last_error(const psr_handle* h) { return h ? h->last_error.c_str() : ""; }

psr_status psr_create(const psr_config* cfg_in, psr_handle** out) {
    if (!out) return PSR_INVALID_INPUT;
    *out = nullptr;
    psr_config cfg;
    if (cfg_in) cfg = *cfg_in;
    else psr_config_default(&cfg);
    if (cfg.max_depth < 2 || cfg.max_depth > kMaxDepth || cfg.max_points <= 0 || cfg.max_triangles <= 0 ||
        cfg.max_mesh_vertices <= 0)
        return PSR_INVALID_INPUT;
    if (cfg.bbox_scale <= 0.0f) cfg.bbox_scale = 1.25f;
    if (cfg.cg_max_iterations <= 0) cfg.cg_max_iterations = 10000;
    psr_handle* h = new (std::nothrow) psr_handle();
    if (!h) return PSR_CUDA_ERROR;
    h->cfg = cfg;
    cudaError_t e = cudaSetDevice(cfg.device);
    if (e != cudaSuccess) { psr_status st = cuda_fail(h, e, "cudaSetDevice"); delete h; return st; }
    Workspace& ws = h->ws;
    memset(&ws, 0, sizeof(ws));
    cudaDeviceGetAttribute(&ws.num_sms, cudaDevAttrMultiProcessorCount, cfg.device);
    if (ws.num_sms <= 0) ws.num_sms = 148;

    const long long N = cfg.max_points;
    const long long nodes = cfg.max_nodes > 0 ? cfg.max_nodes : 10 * N;
    const long long dnodes = std::min(nodes, 8 * N);
    const long long subn = cfg.max_subdivision_nodes > 0 ? cfg.max_subdivision_nodes : 8 * N;
    // live subdivision nodes (all depths) and live depth-D cells: the nodes whose sign is
    // not certain, a small part of the subdivision nodes built
    const long long subd = std::max(65536LL, subn / 4);
    Caps& cap = ws.cap;
    cap.points = (int)N;
    cap.nodes = (int)nodes;
    cap.dnodes = (int)dnodes;
    cap.vertices = (int)std::min(4 * nodes, (long long)1 << 30);
    cap.edges = (int)std::min(6 * dnodes, (long long)1 << 30);
    cap.faces = (int)std::min(4 * nodes, (long long)1 << 30);
    cap.sub_nodes = (int)subn;
    cap.sub_dnodes = (int)subd;
    cap.sub_live = (int)subd;
    cap.mesh_vertices = cfg.max_mesh_vertices;
    cap.mesh_tris = cfg.max_triangles;
    ws.part_cap_v = 2 * cfg.max_mesh_vertices + 4096;
    ws.part_cap_t = 2 * cfg.max_triangles + 4096;
    long long max_scan = std::max({N + 1, nodes, (long long)cap.edges, (long long)cap.faces, (long long)cap.vertices,
                                   subd * 12, (long long)ws.part_cap_v, (long long)ws.part_cap_t,
                                   256LL * ((N + kSortTile - 1) / kSortTile),
                                   (1LL << (3 * kColourGridLevel)) + 1});   // colour cell table
    cap.scan_tiles = (int)((max_scan + kScanMinTile - 1) / kScanMinTile) + 1;
    const int sort_tiles = (int)((N + kSortTile - 1) / kSortTile) + 1;
    const int D = cfg.max_depth;
    ws.res = (1 << (D + 1)) - 1;

    Arena A;
    A.add(ws.cnt, 1);
    A.add(ws.scan.words, (size_t)cap.scan_tiles + kScanHeader);
    A.add(ws.scan_aux.words, (size_t)cap.scan_tiles + kScanHeader);
    A.add(ws.sort.hist, (size_t)kRadix * sort_tiles + 16);
    A.add(ws.sort.keys_alt, (size_t)N);
    A.add(ws.sort.vals_alt, (size_t)N);
    A.add(ws.in_xyz, 3 * (size_t)N);
    A.add(ws.in_nrm, 3 * (size_t)N);
    A.add(ws.in_rgb, 3 * (size_t)N);
    A.add(ws.code, (size_t)N);
    A.add(ws.sidx, (size_t)N);
    A.add(ws.px, (size_t)N); A.add(ws.py, (size_t)N); A.add(ws.pz, (size_t)N);
    A.add(ws.nx, (size_t)N); A.add(ws.ny, (size_t)N); A.add(ws.nz, (size_t)N);
    A.add(ws.cr, (size_t)N); A.add(ws.cg, (size_t)N); A.add(ws.cb, (size_t)N);
    A.add(ws.point2node, (size_t)N);
    A.add(ws.puid, (size_t)N);
    A.add(ws.ucode, (size_t)N);
    A.add(ws.ufirst, (size_t)N + 1);
    A.add(ws.uslot, (size_t)N);
    A.add(ws.uaddr, (size_t)N);
    A.add(ws.tkey, (size_t)nodes); A.add(ws.tpidx, (size_t)nodes); A.add(ws.tpnum, (size_t)nodes);
    A.add(ws.tdidx, (size_t)nodes); A.add(ws.tdnum, (size_t)nodes); A.add(ws.tchild, (size_t)nodes);
    A.add(ws.tparent_slot, (size_t)nodes / 8 + 8);
    A.add(ws.gkey, (size_t)dnodes / 8 + 8); A.add(ws.gpidx, (size_t)dnodes / 8 + 8);
    A.add(ws.gpnum, (size_t)dnodes / 8 + 8); A.add(ws.gdidx, (size_t)dnodes / 8 + 8);
    A.add(ws.gdnum, (size_t)dnodes / 8 + 8); A.add(ws.gaddr, (size_t)dnodes / 8 + 8);
    A.add(ws.key, (size_t)nodes); A.add(ws.pidx, (size_t)nodes); A.add(ws.pnum, (size_t)nodes);
    A.add(ws.parent, (size_t)nodes); A.add(ws.first_child, (size_t)nodes); A.add(ws.didx, (size_t)nodes);
    A.add(ws.dnum, (size_t)nodes); A.add(ws.ndepth, (size_t)nodes); A.add(ws.enc, (size_t)nodes);
    A.add(ws.ctr_x, (size_t)nodes); A.add(ws.ctr_y, (size_t)nodes); A.add(ws.ctr_z, (size_t)nodes);
    A.add(ws.neigh, 27 * (size_t)nodes);
    A.add(ws.node_vtx, 8 * (size_t)nodes);
    A.add(ws.node_edge, 12 * (size_t)nodes);
    A.add(ws.node_face, 6 * (size_t)nodes);
    A.add(ws.dff, (size_t)ws.res * ws.res);
    A.add(ws.stencil, (size_t)(kMaxDepth + 1) * 27);
    A.add(ws.vfield, 3 * (size_t)dnodes);
    A.add(ws.divg, (size_t)nodes);
    A.add(ws.xsol, (size_t)nodes);
    A.add(ws.cg_r, (size_t)nodes); A.add(ws.cg_p, (size_t)nodes); A.add(ws.cg_q, (size_t)nodes);
    A.add(ws.cg_ap, (size_t)nodes);
    A.add(ws.cg_blk, (size_t)nodes * 8 + 64);
    A.add(ws.cg_loop, (size_t)kMaxDepth + 1);
    A.add(ws.cg_loop_part, (size_t)(kMaxDepth + 1) * kLoopMaxBlocks);
    A.add(ws.cg_loop_ctl, (size_t)kLoopControlWords);
    A.add(ws.cg_partial, std::max((size_t)nodes, (size_t)4096 * (kMaxDepth + 1)));
    A.add(ws.point_val, (size_t)N);
    A.add(ws.pv_coef, 27 * ((size_t)dnodes / 8 + 64));
    A.add(ws.iso_partial, (size_t)N / kBlock + 2);   // one sum per chunk of kBlock sample points
    A.add(ws.vmask, (size_t)nodes);
    A.add(ws.emask16, (size_t)dnodes);
    A.add(ws.fmask, (size_t)nodes);
    A.add(ws.v_x, (size_t)cap.vertices); A.add(ws.v_y, (size_t)cap.vertices); A.add(ws.v_z, (size_t)cap.vertices);
    A.add(ws.v_owner, (size_t)cap.vertices); A.add(ws.v_kind, (size_t)cap.vertices); A.add(ws.v_depth, (size_t)cap.vertices);
    A.add(ws.e_owner, (size_t)cap.edges); A.add(ws.e_kind, (size_t)cap.edges);
    A.add(ws.f_owner, (size_t)cap.faces); A.add(ws.f_kind, (size_t)cap.faces); A.add(ws.f_hasparent, (size_t)cap.faces);
    A.add(ws.vvalue, (size_t)cap.vertices);
    A.add(ws.e_cross, (size_t)cap.edges);
    A.add(ws.cube_class, (size_t)dnodes);
    A.add(ws.face_hit, (size_t)cap.faces);
    A.add(ws.sub_root, (size_t)nodes);
    A.add(ws.sub_root_depth, (size_t)nodes);
    A.add(ws.root_group, (size_t)nodes);
    A.add(ws.root_self, (size_t)nodes);
    // roots beyond this capacity take the walk over their octree chain in the subdivision
    // scan itself; psr_config.root_poly_capacity sets it (that path gives the same mesh)
    ws.cap_poly = (int)std::max<long long>(65536, nodes / 16);
    if (cfg.root_poly_capacity > 0) ws.cap_poly = cfg.root_poly_capacity;
    A.add(ws.root_poly, 28 * (size_t)ws.cap_poly);
    A.add(ws.c_vnode, (size_t)subn); A.add(ws.c_key, (size_t)subn); A.add(ws.c_group, (size_t)subn);
    A.add(ws.c_parent, (size_t)subn); A.add(ws.c_jump, (size_t)subn); A.add(ws.c_depth, (size_t)subn);
    A.add(ws.c_cx, (size_t)subn); A.add(ws.c_cy, (size_t)subn); A.add(ws.c_cz, (size_t)subn);
    A.add(ws.c_neigh, 27 * (size_t)subn);
    A.add(ws.c_live, (size_t)subd);
    A.add(ws.c_poly, 28 * (size_t)subd);
    A.add(ws.c_touch, (size_t)subd);
    A.add(ws.lv_vnode, (size_t)subd);
    A.add(ws.lv_nb, 27 * (size_t)subd);
    A.add(ws.s_vtx, 8 * (size_t)subd); A.add(ws.s_edge, 12 * (size_t)subd);
    A.add(ws.s_vmask, (size_t)subd); A.add(ws.s_emask, (size_t)subd);
    A.add(ws.sv_x, 8 * (size_t)subd); A.add(ws.sv_y, 8 * (size_t)subd); A.add(ws.sv_z, 8 * (size_t)subd);
    A.add(ws.sv_owner, 8 * (size_t)subd); A.add(ws.sv_kind, 8 * (size_t)subd); A.add(ws.sv_value, 8 * (size_t)subd);
    A.add(ws.se_owner, 12 * (size_t)subd); A.add(ws.se_kind, 12 * (size_t)subd); A.add(ws.se_cross, 12 * (size_t)subd);
    A.add(ws.s_cube_class, (size_t)subd);
    A.add(ws.mesh_v, 3 * (size_t)cap.mesh_vertices);
    A.add(ws.mesh_t, 3 * (size_t)cap.mesh_tris);
    A.add(ws.mesh_c, 3 * (size_t)cap.mesh_vertices);
    A.add(ws.mesh_n, 3 * (size_t)cap.mesh_vertices);
    A.add(ws.nacc, 3 * (size_t)cap.mesh_vertices);
    A.add(ws.vcount, (size_t)cap.mesh_vertices);
    A.add(ws.cell_start, ((size_t)1 << (3 * kColourGridLevel)) + 16);
    A.add(ws.colour_far, 2 * (size_t)cap.mesh_vertices);
    A.add(ws.colour_far2, 2 * (size_t)cap.mesh_vertices);
    if (cfg.weld_vertices) {
        size_t slots = 1;
        while (slots < 2 * (size_t)cap.mesh_vertices) slots <<= 1;
        ws.weld_mask = (unsigned)(slots - 1);
        A.add(ws.weld_table, slots);
        A.add(ws.weld_slot, (size_t)cap.mesh_vertices);
        A.add(ws.weld_newid, (size_t)cap.mesh_vertices);
        A.add(ws.weld_v, 3 * (size_t)cap.mesh_vertices);
    }
    A.add(ws.part_v, 3 * (size_t)ws.part_cap_v);
    A.add(ws.part_t, 3 * (size_t)ws.part_cap_t);
    ws.mb.max_groups = (int)nodes;
    A.add(ws.mb.ov_group, 8 * (size_t)nodes);
    A.add(ws.mb.ov_sub, 8 * (size_t)nodes);
    A.add(ws.mb.groups, 8 * (size_t)nodes);
    A.add(ws.mb.edge_of_dnode, (size_t)subd);
    A.add(ws.mb.tri_of_dnode, (size_t)subd);
    A.add(ws.mb.group_cross0, (size_t)nodes);
    A.add(ws.mb.parts, 4 * (size_t)nodes + 8);
    A.add(ws.mb.kept_prefix, (size_t)ws.part_cap_v);
    A.add(ws.mb.misc, 16);
    A.add(ws.d_params, 16);

    if (cfg.batch_clouds > kMaxBatchClouds || cfg.cg_cluster_ctas < 0 || cfg.cg_cluster_ctas > 16 ||
        cfg.cg_cluster_ctas_fine < 0 || cfg.cg_cluster_ctas_fine > 16) {
        delete h;
        return PSR_INVALID_INPUT;
    }
    h->clouds = cfg.batch_clouds > 1 ? cfg.batch_clouds : 1;
    if (h->clouds == 1) {
        e = cudaMalloc(&h->arena, A.bytes);
        if (e != cudaSuccess) { psr_status st = cuda_fail(h, e, "cudaMalloc workspace"); delete h; return st; }
    } else {
        const psr_status st = map_cloud_slots(h, A.bytes);
        if (st != PSR_OK) { delete h; return st; }
        h->arena = (void*)h->va_base;
    }
    h->arena_bytes = A.bytes;
    A.assign((char*)h->arena);
    set_batch(ws, 1);
    ws.cg_ctas = cfg.cg_cluster_ctas;
    ws.cg_ctas_fine = cfg.cg_cluster_ctas_fine;
    ws.scan.max_tiles = cap.scan_tiles;
    // scan counters and epoch start at zero; the scans keep them consistent afterwards
    e = cudaMemset(ws.scan.words, 0, sizeof(unsigned long long) * ((size_t)cap.scan_tiles + kScanHeader));
    ws.scan_aux.max_tiles = cap.scan_tiles;
    if (e == cudaSuccess)
        e = cudaMemset(ws.scan_aux.words, 0, sizeof(unsigned long long) * ((size_t)cap.scan_tiles + kScanHeader));
    // the device-loop CG's block tickets start at zero; each reduction leaves them at zero
    if (e == cudaSuccess) e = cudaMemset(ws.cg_loop, 0, sizeof(CgLoopState) * (kMaxDepth + 1));
    ws.sort.max_tiles = sort_tiles;
    ws.sort.scan = ws.scan;   // sort shares the scan scratch (scans are sequential on one stream)
    e = cudaMallocHost(&h->cnt_host_all, sizeof(Counters) * (size_t)h->clouds);
    ws.cnt_host = h->cnt_host_all;
    if (e == cudaSuccess) e = cudaMallocHost(&h->h_params, 16 * sizeof(int) * (size_t)h->clouds);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking);
    for (int i = 0; i < 7 && e == cudaSuccess; ++i) e = cudaEventCreate(&h->ev[i]);
    h->ws.ev_cg = h->ev[6];
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ws.aux, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ws.ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ws.ev_join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ws.aux2, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ws.ev_fork2, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ws.ev_join2, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ws.aux3, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ws.ev_join3, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ws.aux4, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ws.ev_join4, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ws.loop_body, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->done, cudaEventDisableTiming);
    // tables
    if (e == cudaSuccess) e = upload_tables_octree();
    if (e == cudaSuccess) e = upload_tables_field();
    if (e == cudaSuccess) e = upload_tables_solver();
    if (e == cudaSuccess) e = upload_tables_mesh();
    if (e == cudaSuccess) e = upload_tables_transfer();
    if (e == cudaSuccess) {
        std::vector<double> dff;
        build_dff_table(D, dff);
        std::vector<float> st;
        build_stencil(kMaxDepth, st, (double)cfg.laplacian_epsilon);
        std::vector<float> dff32(dff.begin(), dff.end());   // the kernels use float entries
        e = cudaMemcpy(ws.dff, dff32.data(), dff32.size() * sizeof(float), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(ws.stencil, st.data(), st.size() * sizeof(float), cudaMemcpyHostToDevice);
        std::copy(st.begin(), st.end(), ws.stencil_host);   // the CG launch passes some as parameters
    }
    // the other cloud slots start as copies of slot 0 (tables, zeroed scan counters)
    for (int k = 1; k < h->clouds && e == cudaSuccess; ++k)
        e = cudaMemcpy(slot_ptr((char*)h->arena, k), h->arena, A.bytes, cudaMemcpyDeviceToDevice);
    // device-to-device copies and memsets return before they complete, and the handle's
    // streams do not wait for the legacy default stream: finish the set-up here, so no
    // later copy into a slot can be overwritten by it
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) {
        prepare_launch_configs(ws);
        e = cudaGetLastError();
    }
    if (cfg.disable_graphs) h->use_graphs = 0;
    if (e != cudaSuccess) {
        psr_status st = cuda_fail(h, e, "psr_create");
        psr_destroy(h);
        return st;
    }
    *out = h;
    return PSR_OK;
}

psr_status psr_destroy(psr_handle* h) {
    if (!h) return PSR_OK;
    if (h->pending && h->done) cudaEventSynchronize(h->done);   // no buffer is freed under running work
    // work a failed call left queued may still run: unmapping a batch handle's slots (unlike
    // cudaFree) does not wait for it
    if (h->va_base) cudaDeviceSynchronize();
    for (auto& g : h->graphs) if (g.second.exec) cudaGraphExecDestroy(g.second.exec);
    if (h->arena && h->clouds == 1) cudaFree(h->arena);
    if (h->va_base) release_cloud_slots(h, h->clouds);
    if (h->cnt_host_all) cudaFreeHost(h->cnt_host_all);
    if (h->h_params) cudaFreeHost(h->h_params);
    for (int i = 0; i < 7; ++i) if (h->ev[i]) cudaEventDestroy(h->ev[i]);
    if (h->ws.ev_fork) cudaEventDestroy(h->ws.ev_fork);
    if (h->ws.ev_join) cudaEventDestroy(h->ws.ev_join);
    if (h->ws.ev_fork2) cudaEventDestroy(h->ws.ev_fork2);
    if (h->ws.ev_join2) cudaEventDestroy(h->ws.ev_join2);
    if (h->ws.ev_join3) cudaEventDestroy(h->ws.ev_join3);
    if (h->ws.ev_join4) cudaEventDestroy(h->ws.ev_join4);
    if (h->ws.aux4) cudaStreamDestroy(h->ws.aux4);
    if (h->ws.loop_body) cudaStreamDestroy(h->ws.loop_body);
    if (h->ws.aux3) cudaStreamDestroy(h->ws.aux3);
    if (h->ws.aux2) cudaStreamDestroy(h->ws.aux2);
    if (h->ws.aux) cudaStreamDestroy(h->ws.aux);
    if (h->done) cudaEventDestroy(h->done);
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
    delete h;
    return PSR_OK;
}

// copies the mesh of the last run into device-resident caller buffers (counts read on the
// device, clamped to the caller's capacities), so a device-output call needs no host wait
__global__ void __launch_bounds__(kBlock) k_emit_mesh(const Counters* c, const float* v, const int* t,
                                                      const float* col, const float* nrm, float* ov, int* ot,
                                                      float* oc, float* on, int vcap, int tcap) {
    const int nv = 3 * min(max(c->n_mesh_vertices, 0), vcap);
    const int nt = 3 * min(max(c->n_mesh_triangles, 0), tcap);
    PSR_GRID_STRIDE(i, max(nv, nt)) {
        if (i < nv) {
            if (ov) ov[i] = v[i];
            if (oc) oc[i] = col[i];
            if (on) on[i] = nrm[i];
        }
        if (i < nt && ot) ot[i] = t[i];
    }
}

// The whole pipeline for the clouds set by set_batch, issued on `qs` (captured into a graph
// or run directly).
#ifdef PSR_CLOUD_CHECK
#define PSR_TRACE(q, what) do { if ((q) != cudaSuccess) fprintf(stderr, "issue_pipeline: %s: %s\n", what, cudaGetErrorString(q)); } while (0)
#else
#define PSR_TRACE(q, what) do { } while (0)
#endif

static cudaError_t issue_pipeline(psr_handle* h, cudaStream_t qs, int cg_iters, int want_colour, int want_normals) {
    Workspace& ws = h->ws;
    ws.stream = qs;
    // stage-boundary events: external event nodes when captured into a graph (so a replay
    // records them), plain records when the stages are issued directly (the external flag
    // is refused outside a capture)
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(qs, &cap);
    ws.ev_flags = (cap == cudaStreamCaptureStatusActive) ? cudaEventRecordExternal : cudaEventRecordDefault;
    cudaError_t q = cudaEventRecordWithFlags(h->ev[0], qs, ws.ev_flags);
    PSR_TRACE(q, "event 0");
    if (q == cudaSuccess) q = octree_build(ws); PSR_TRACE(q, "octree_build");
    if (q == cudaSuccess) q = cudaEventRecordWithFlags(h->ev[1], qs, ws.ev_flags);
    // octree-only work on a third stream, beside the divergence and the solve: the
    // vertex / edge / face records and the colour search grid (own scan scratch)
    const bool overlap = h->cfg.concurrent_stages != 0;
    if (overlap) {
        if (q == cudaSuccess) q = cudaEventRecord(ws.ev_fork2, qs);
        if (q == cudaSuccess) q = cudaStreamWaitEvent(ws.aux2, ws.ev_fork2, 0);
        if (q == cudaSuccess) {
            const ScanScratch main_scan = ws.scan;
            ws.stream = ws.aux2;
            ws.scan = ws.scan_aux;
            q = mesh_geometry(ws);
            if (q == cudaSuccess) q = transfer_prepare(ws, want_colour); PSR_TRACE(q, "mesh_geometry/transfer_prepare");
            ws.stream = qs;
            ws.scan = main_scan;
        }
        if (q == cudaSuccess) q = cudaEventRecord(ws.ev_join2, ws.aux2);
    } else {
        if (q == cudaSuccess) q = mesh_geometry(ws);
        if (q == cudaSuccess) q = transfer_prepare(ws, want_colour);
    }
    if (q == cudaSuccess) q = field_build(ws); PSR_TRACE(q, "field_build");
    if (q == cudaSuccess) q = cudaEventRecordWithFlags(h->ev[2], qs, ws.ev_flags);
    if (q == cudaSuccess)
        q = solve_build(ws, cg_iters > 0 ? 1 : 0, cg_iters, h->cfg.cg_tolerance, h->cfg.cg_max_iterations,
                        h->cfg.cg_residual_period == 0 ? kDefaultResidualPeriod
                                                       : (h->cfg.cg_residual_period < 0 ? -1 : h->cfg.cg_residual_period)); PSR_TRACE(q, "solve_build");
    if (q == cudaSuccess) q = cudaEventRecordWithFlags(h->ev[3], qs, ws.ev_flags);
    if (q == cudaSuccess && overlap) q = cudaStreamWaitEvent(qs, ws.ev_join2, 0);
    if (q == cudaSuccess) q = mesh_build(ws); PSR_TRACE(q, "mesh_build");
    if (q == cudaSuccess) q = weld_build(ws); PSR_TRACE(q, "weld_build");
    if (q == cudaSuccess) q = cudaEventRecordWithFlags(h->ev[4], qs, ws.ev_flags);
    if (q == cudaSuccess) q = transfer_build(ws, want_colour, want_normals); PSR_TRACE(q, "transfer_build");
    if (q == cudaSuccess) q = cudaEventRecordWithFlags(h->ev[5], qs, ws.ev_flags);
    return q;
}

// Launches the pipeline for `clouds` clouds (slots 0 .. clouds - 1) on `s`: captured once
// per (clouds, depth, options) into a CUDA graph, replayed afterwards.
static cudaError_t launch_pipeline(psr_handle* h, int depth, int cg_iters, int want_colour, int want_normals,
                                   bool has_rgb, int clouds, cudaStream_t s) {
    Workspace& ws = h->ws;
    ws.depth = depth;
    uint8_t* saved_rgb = ws.in_rgb;
    if (!has_rgb) ws.in_rgb = nullptr;
    set_batch(ws, clouds);
    cudaError_t e = cudaSuccess;
    const long long gkey = ((long long)clouds << 44) | ((long long)depth << 40) | ((long long)cg_iters << 8) |
                           (want_colour << 2) | (want_normals << 1) | (has_rgb ? 1 : 0);
    h->last_graph = 0;
    if (h->use_graphs) {
        auto it = h->graphs.find(gkey);
        if (it == h->graphs.end()) {
            cudaGraph_t graph = nullptr;
            GraphEntry ge;
            cudaError_t q = cudaStreamBeginCapture(h->own_stream, cudaStreamCaptureModeThreadLocal);
            if (q == cudaSuccess) {
                cudaError_t qi = issue_pipeline(h, h->own_stream, cg_iters, want_colour, want_normals);
                q = cudaStreamEndCapture(h->own_stream, &graph);
                if (qi != cudaSuccess) q = qi;
            }
            if (q == cudaSuccess) q = cudaGraphInstantiate(&ge.exec, graph, 0);
            if (q == cudaSuccess) {
                size_t nn = 0;
                cudaGraphGetNodes(graph, nullptr, &nn);
                std::vector<cudaGraphNode_t> nodes(nn);
                cudaGraphGetNodes(graph, nodes.data(), &nn);
                for (auto nd : nodes) {
                    cudaGraphNodeType t;
                    if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ge.kernels++;
                }
            }
            if (graph) cudaGraphDestroy(graph);
            if (q != cudaSuccess) {
                (void)cudaGetLastError();
                h->use_graphs = 0;   // capture not available: run the stages directly from now on
                if (ge.exec) cudaGraphExecDestroy(ge.exec);
            } else {
                it = h->graphs.emplace(gkey, ge).first;
            }
        }
        if (h->use_graphs) {
            e = cudaGraphLaunch(it->second.exec, s);
            h->last_kernels = it->second.kernels;
            h->last_graph = 1;
        }
    }
    if (!h->use_graphs) {
        e = issue_pipeline(h, s, cg_iters, want_colour, want_normals);
        h->last_kernels = -1;
    }
    set_batch(ws, 1);
    ws.in_rgb = saved_rgb;
    ws.stream = s;
    return e;
}

// Copies the inputs of one cloud into slot k and enqueues its point count.
static cudaError_t stage_inputs(psr_handle* h, const psr_points* pts, int k, cudaStream_t s) {
    Workspace& ws = h->ws;
    const int n = pts->count;
    const cudaMemcpyKind kind = (pts->location == PSR_DEVICE) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    cudaError_t e = cudaMemcpyAsync(slot_ptr(ws.in_xyz, k), pts->xyz, 3 * sizeof(float) * (size_t)n, kind, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(slot_ptr(ws.in_nrm, k), pts->normals, 3 * sizeof(float) * (size_t)n, kind, s);
    if (e == cudaSuccess && pts->rgb) e = cudaMemcpyAsync(slot_ptr(ws.in_rgb, k), pts->rgb, 3 * (size_t)n, kind, s);
    if (e == cudaSuccess) {
        int* hp = h->h_params + 16 * k;
        hp[0] = n;
        e = cudaMemcpyAsync(slot_ptr(ws.d_params, k), hp, sizeof(int), cudaMemcpyHostToDevice, s);
    }
    return e;
}

// Device address of a host output buffer the GPU can write (pinned or registered host
// memory), else nullptr.  NULL stays NULL (output not asked for).
static void* device_view(void* p, bool& ok) {
    if (!p) return nullptr;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        (void)cudaGetLastError();
        ok = false;
        return nullptr;
    }
    if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) return p;
    if (at.type == cudaMemoryTypeHost && at.devicePointer) return at.devicePointer;
    ok = false;
    return nullptr;
}

// Enqueues the count read-back of slot k and the copy of its mesh into the caller's
// buffers by a kernel that reads the counts on the device (no host wait): for device
// outputs, and for host outputs in pinned or registered memory, which the kernel writes
// through their device addresses.  Other host outputs are copied when the work has
// completed (*emitted = false).
static cudaError_t stage_outputs(psr_handle* h, psr_mesh* mesh, int k, int want_colour, int want_normals,
                                 cudaStream_t s, bool* emitted) {
    Workspace& ws = h->ws;
    cudaError_t e =
        cudaMemcpyAsync(h->cnt_host_all + k, slot_ptr(ws.cnt, k), sizeof(Counters), cudaMemcpyDeviceToHost, s);
    bool ok = true;
    void* dv = device_view(mesh->vertices, ok);
    void* dt = device_view(mesh->triangles, ok);
    void* dc = want_colour ? device_view(mesh->colors, ok) : nullptr;
    void* dn = want_normals ? device_view(mesh->normals, ok) : nullptr;
    *emitted = ok;
    if (e == cudaSuccess && ok) {
        k_emit_mesh<<<ws.num_sms * 4, kBlock, 0, s>>>(slot_ptr(ws.cnt, k), slot_ptr(ws.mesh_v, k),
                                                      slot_ptr(ws.mesh_t, k), slot_ptr(ws.mesh_c, k),
                                                      slot_ptr(ws.mesh_n, k), (float*)dv, (int*)dt, (float*)dc,
                                                      (float*)dn, mesh->vertex_capacity, mesh->triangle_capacity);
        e = cudaGetLastError();
    }
    return e;
}

static psr_status check_points(psr_handle* h, const psr_points* pts, const psr_mesh* mesh) {
    if (!pts || !mesh || !pts->xyz || !pts->normals) return fail(h, PSR_INVALID_INPUT, "null argument");
    if (pts->count <= 0) return fail(h, PSR_INVALID_INPUT, "empty point cloud");
    if (pts->count > h->ws.cap.points) return fail(h, PSR_OUT_OF_CAPACITY, "more points than max_points");
    return PSR_OK;
}

// Enqueues the reconstruction of `count` clouds (one launch per kernel for all of them) on
// `stream`, without a host synchronisation.  psr_submit is the one-cloud case.
static psr_status submit_clouds(psr_handle* h, const psr_points* pts, int count, const psr_options* opt,
                                psr_mesh* meshes, void* stream, bool batch_call) {
    if (h->pending) return fail(h, PSR_INVALID_INPUT, "a reconstruction is already in flight on this handle");
    h->have_result = false;
    h->batch_stats.clear();
    h->batch_status.clear();
    if (!pts || !meshes || count < 1) return fail(h, PSR_INVALID_INPUT, "null argument or no cloud");
    if (count > h->clouds) return fail(h, PSR_OUT_OF_CAPACITY, "more clouds than the handle's batch_clouds");
    for (int k = 0; k < count; ++k) {
        const psr_status st = check_points(h, pts + k, meshes + k);
        if (st != PSR_OK) return st;
    }
    const bool has_rgb = pts[0].rgb != nullptr;
    const int want_colour = h->cfg.compute_colors && meshes[0].colors;
    const int want_normals = h->cfg.compute_normals && meshes[0].normals;
    for (int k = 1; k < count; ++k)
        if ((pts[k].rgb != nullptr) != has_rgb || (h->cfg.compute_colors && meshes[k].colors) != want_colour ||
            (h->cfg.compute_normals && meshes[k].normals) != want_normals)
            return fail(h, PSR_INVALID_INPUT, "the clouds of a batch differ in colour or normal outputs");
    const int depth = (opt && opt->depth > 0) ? opt->depth : h->cfg.max_depth;
    if (depth < 2 || depth > h->cfg.max_depth) return fail(h, PSR_INVALID_INPUT, "depth outside [2, max_depth]");
    const int cg_iters = (opt && opt->cg_iterations > 0) ? opt->cg_iterations : 0;
    cudaStream_t s = stream ? (cudaStream_t)stream : h->own_stream;
    cudaError_t e = cudaSetDevice(h->cfg.device);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaSetDevice");
    for (int k = 0; k < count && e == cudaSuccess; ++k) e = stage_inputs(h, pts + k, k, s);
    if (e != cudaSuccess) return cuda_fail(h, e, "input copy");
    e = launch_pipeline(h, depth, cg_iters, want_colour, want_normals, has_rgb, count, s);
    h->pend_emitted.assign(count, 0);
    for (int k = 0; k < count && e == cudaSuccess; ++k) {
        bool em = false;
        e = stage_outputs(h, meshes + k, k, want_colour, want_normals, s, &em);
        h->pend_emitted[k] = em;
    }
    if (e == cudaSuccess) e = cudaEventRecord(h->done, s);
    if (e != cudaSuccess) return cuda_fail(h, e, "reconstruct");
    h->pending = true;
    h->pend_meshes.assign(meshes, meshes + count);
    h->pend_batch = batch_call;
    h->pend_depth = depth;
    h->pend_colour = want_colour;
    h->pend_normals = want_normals;
    h->pend_stream = s;
    return PSR_OK;
}

static psr_status status_of(const Counters& c) {
    if (c.error & kErrInvalid) return PSR_INVALID_INPUT;
    if (c.error & kErrCapacity) return PSR_OUT_OF_CAPACITY;
    if (c.error & kErrSpinTimeout) return PSR_DEVICE_TIMEOUT;
    return PSR_OK;
}

static const char* status_message(psr_status st) {
    switch (st) {
        case PSR_INVALID_INPUT: return "non-finite input or malformed octree";
        case PSR_OUT_OF_CAPACITY: return "a device count exceeded its capacity";
        case PSR_DEVICE_TIMEOUT: return "a bounded device wait gave up";
        default: return "";
    }
}

static void fill_stats(const psr_handle* h, const Counters& c, int depth, psr_stats& st) {
    memset(&st, 0, sizeof(st));
    st.points = c.n_points; st.unique_leaves = c.n_unique; st.nodes = c.n_nodes; st.depth = depth;
    for (int d = 0; d <= kMaxDepth; ++d) {
        st.level_count[d] = c.level_count[d];
        st.cg_iterations[d] = c.cg_iters[d];
        st.cg_residual[d] = c.cg_rr[d] > 0 ? sqrt(c.cg_rr[d]) : 0.0;
        st.cg_true_residual[d] = c.cg_rr_true[d] >= 0 ? sqrt(c.cg_rr_true[d]) : -1.0;
        st.cg_residual_checks[d] = c.cg_checks[d];
        st.cg_restarts[d] = c.cg_restarts[d];
        st.cg_depth_ms[d] = (float)(c.cg_depth_ns[d] * 1e-6);
    }
    st.vertices = c.n_vertices; st.edges = c.n_edges; st.faces = c.n_faces;
    st.crossings = c.n_cross; st.triangles = c.n_tri;
    st.subdivision_roots = c.n_subroots; st.subdivision_nodes = c.n_sub_nodes;
    st.mesh_vertices = c.n_mesh_vertices; st.mesh_triangles = c.n_mesh_triangles;
    st.iso_value = c.iso;
    st.error_bits = c.error;
    st.kernel_launches = h->last_kernels;
    st.graph_replay = h->last_graph;
    for (int i = 0; i < 5; ++i) cudaEventElapsedTime(&st.stage_ms[i], h->ev[i], h->ev[i + 1]);
    cudaEventElapsedTime(&st.stage_ms[5], h->ev[0], h->ev[5]);
    cudaEventElapsedTime(&st.cg_kernel_ms, h->ev[2], h->ev[6]);
}

// Mesh counts and, for host outputs, the copies of cloud k (after its work completed).
static psr_status finish_cloud(psr_handle* h, int k, const Counters& c, psr_status st) {
    Workspace& ws = h->ws;
    psr_mesh* mesh = &h->pend_meshes[k];
    cudaStream_t s = h->pend_stream;
    if (st != PSR_OK) return st;
    mesh->vertex_count = c.n_mesh_vertices;
    mesh->triangle_count = c.n_mesh_triangles;
    for (int a = 0; a < 3; ++a) mesh->center[a] = c.center[a];
    mesh->scale = c.max_edge;
    if (c.n_mesh_vertices > mesh->vertex_capacity || c.n_mesh_triangles > mesh->triangle_capacity) {
        h->last_error = "output mesh buffers too small";
        return PSR_OUT_OF_CAPACITY;
    }
    if (h->pend_emitted[k]) return PSR_OK;   // written by k_emit_mesh
    const cudaMemcpyKind ok = cudaMemcpyDeviceToHost;
    cudaError_t e = cudaSuccess;
    if (mesh->vertices && c.n_mesh_vertices)
        e = cudaMemcpyAsync(mesh->vertices, slot_ptr(ws.mesh_v, k), 3 * sizeof(float) * (size_t)c.n_mesh_vertices, ok, s);
    if (e == cudaSuccess && mesh->triangles && c.n_mesh_triangles)
        e = cudaMemcpyAsync(mesh->triangles, slot_ptr(ws.mesh_t, k), 3 * sizeof(int) * (size_t)c.n_mesh_triangles, ok, s);
    if (e == cudaSuccess && h->pend_colour && c.n_mesh_vertices)
        e = cudaMemcpyAsync(mesh->colors, slot_ptr(ws.mesh_c, k), 3 * sizeof(float) * (size_t)c.n_mesh_vertices, ok, s);
    if (e == cudaSuccess && h->pend_normals && c.n_mesh_vertices)
        e = cudaMemcpyAsync(mesh->normals, slot_ptr(ws.mesh_n, k), 3 * sizeof(float) * (size_t)c.n_mesh_vertices, ok, s);
    return e == cudaSuccess ? PSR_OK : PSR_CUDA_ERROR;
}

// After the submitted work has completed: statistics, status, mesh counts, host copies.
static psr_status complete_impl(psr_handle* h) {
    h->pending = false;
    const int count = (int)h->pend_meshes.size();
    h->batch_stats.assign(count, psr_stats{});
    h->batch_status.assign(count, PSR_OK);
    psr_status first = PSR_OK;
    for (int k = 0; k < count; ++k) {
        const Counters& c = h->cnt_host_all[k];
        fill_stats(h, c, h->pend_depth, h->batch_stats[k]);
        const psr_status st = finish_cloud(h, k, c, status_of(c));
        h->batch_status[k] = st;
        if (st != PSR_OK && first == PSR_OK) first = st;
    }
    bool copies = false;
    for (int k = 0; k < count; ++k) copies = copies || (!h->pend_emitted[k] && h->batch_status[k] == PSR_OK);
    const cudaError_t e = copies ? cudaStreamSynchronize(h->pend_stream) : cudaSuccess;   // the host copies
    if (h->pend_batch) {
        for (int k = 0; k < count; ++k) h->pend_user_meshes[k] = h->pend_meshes[k];
    } else {
        // one-cloud call: its results are the handle's (stats, debug arrays)
        h->host_cnt = h->cnt_host_all[0];
        h->stats = h->batch_stats[0];
        h->have_result = true;
        *h->pend_user_mesh = h->pend_meshes[0];
    }
    if (e != cudaSuccess) return cuda_fail(h, e, "output copy");
    if (first == PSR_OK) return PSR_OK;
    if (h->pend_batch) return fail(h, first, "a cloud of the batch failed (see psr_get_batch_result)");
    if (status_of(h->cnt_host_all[0]) != PSR_OK) return fail(h, first, status_message(first));
    return first;   // the output buffers were too small (message set by finish_cloud)
}

psr_status psr_reconstruct(psr_handle* h, const psr_points* pts, const psr_options* opt, psr_mesh* mesh,
                           void* stream) {
    psr_status st = psr_submit(h, pts, opt, mesh, stream);
    if (st != PSR_OK) return st;
    return psr_wait(h);
}

psr_status psr_submit(psr_handle* h, const psr_points* pts, const psr_options* opt, psr_mesh* mesh, void* stream) {
    if (!h) return PSR_INVALID_INPUT;
    if (!mesh) return fail(h, PSR_INVALID_INPUT, "null argument");
    const psr_status st = submit_clouds(h, pts, 1, opt, mesh, stream, false);
    if (st == PSR_OK) h->pend_user_mesh = mesh;
    return st;
}

psr_status psr_submit_batch(psr_handle* h, const psr_points* points, int count, const psr_options* options,
                            psr_mesh* meshes, void* stream) {
    if (!h) return PSR_INVALID_INPUT;
    const psr_status st = submit_clouds(h, points, count, options, meshes, stream, true);
    if (st == PSR_OK) h->pend_user_meshes = meshes;
    return st;
}

psr_status psr_reconstruct_batch(psr_handle* h, const psr_points* points, int count, const psr_options* options,
                                 psr_mesh* meshes, void* stream) {
    psr_status st = psr_submit_batch(h, points, count, options, meshes, stream);
    if (st != PSR_OK) return st;
    return psr_wait(h);
}

psr_status psr_get_batch_result(const psr_handle* h, int index, psr_stats* out) {
    if (!h || index < 0 || index >= (int)h->batch_status.size()) return PSR_INVALID_INPUT;
    if (out) *out = h->batch_stats[index];
    return h->batch_status[index];
}

psr_status psr_poll(psr_handle* h) {
    if (!h) return PSR_INVALID_INPUT;
    if (!h->pending) return fail(h, PSR_INVALID_INPUT, "no reconstruction in flight");
    const cudaError_t q = cudaEventQuery(h->done);
    if (q == cudaErrorNotReady) return PSR_PENDING;
    if (q != cudaSuccess) {
        h->pending = false;
        return cuda_fail(h, q, "reconstruct");
    }
    return complete_impl(h);
}

psr_status psr_wait(psr_handle* h) {
    if (!h) return PSR_INVALID_INPUT;
    if (!h->pending) return fail(h, PSR_INVALID_INPUT, "no reconstruction in flight");
    const cudaError_t q = cudaEventSynchronize(h->done);
    if (q != cudaSuccess) {
        h->pending = false;
        return cuda_fail(h, q, "reconstruct");
    }
    return complete_impl(h);
}

psr_status psr_estimate_normals(psr_handle* h, const float* xyz, int count, psr_location location, float* normals,
                                const float* viewpoint, void* stream) {
    if (!h) return PSR_INVALID_INPUT;
    if (count < 0 || (count > 0 && (!xyz || !normals))) return fail(h, PSR_INVALID_INPUT, "bad arguments");
    if (h->pending) return fail(h, PSR_INVALID_INPUT, "a reconstruction is in flight on this handle");
    if (count > h->ws.cap.points) return fail(h, PSR_OUT_OF_CAPACITY, "more points than max_points");
    // the 10 neighbours of every point are kept in the node neighbour table's storage
    if ((size_t)27 * h->ws.cap.nodes < (size_t)10 * count)
        return fail(h, PSR_OUT_OF_CAPACITY, "max_nodes too small for the neighbour lists");
    if (count == 0) return PSR_OK;
    Workspace& ws = h->ws;
    cudaStream_t s = stream ? (cudaStream_t)stream : h->own_stream;
    ws.stream = s;
    h->have_result = false;   // the stage reuses the reconstruction's scratch
    const float vp[3] = {viewpoint ? viewpoint[0] : 0.0f, viewpoint ? viewpoint[1] : 0.0f,
                         viewpoint ? viewpoint[2] : 0.0f};
    const size_t bytes = 3 * sizeof(float) * (size_t)count;
    const float* in = xyz;
    float* out = normals;
    cudaError_t e = cudaSuccess;
    if (location == PSR_HOST) {
        e = cudaMemcpyAsync(ws.in_xyz, xyz, bytes, cudaMemcpyHostToDevice, s);
        in = ws.in_xyz;
        out = ws.in_nrm;
    }
    if (e == cudaSuccess) e = normals_build(ws, in, count, out, vp[0], vp[1], vp[2]);
    if (e == cudaSuccess && location == PSR_HOST) e = cudaMemcpyAsync(normals, out, bytes, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ws.cnt_host, ws.cnt, sizeof(Counters), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(h, e, "normal estimation");
    const unsigned err = ws.cnt_host->error;
    if (err & kErrInvalid) return fail(h, PSR_INVALID_INPUT, "non-finite input coordinates");
    if (err & kErrCapacity) return fail(h, PSR_OUT_OF_CAPACITY, "a device count exceeded its capacity");
    if (err & kErrSpinTimeout) return fail(h, PSR_DEVICE_TIMEOUT, "a bounded device wait gave up");
    return PSR_OK;
}

psr_status psr_memory_bytes(const psr_handle* h, size_t* bytes) {
    if (!h || !bytes) return PSR_INVALID_INPUT;
    *bytes = h->arena_bytes * (size_t)h->clouds;
    return PSR_OK;
}

psr_status psr_get_stats(const psr_handle* h, psr_stats* out) {
    if (!h || !out) return PSR_INVALID_INPUT;
    *out = h->stats;
    return PSR_OK;
}

psr_status psr_debug_array(psr_handle* h, const char* name, void* dst, size_t dst_bytes, size_t* bytes) {
    if (!h || !name) return PSR_INVALID_INPUT;
    // "name@k": the array of cloud k of the last multi-cloud call
    std::string nm(name);
    int slot = -1;
    const size_t at = nm.find('@');
    if (at != std::string::npos) {
        slot = atoi(nm.c_str() + at + 1);
        nm = nm.substr(0, at);
        if (slot < 0 || slot >= (int)h->batch_stats.size() || slot >= h->clouds || h->pending)
            return fail(h, PSR_INVALID_INPUT, "no such cloud in the last call");
    } else if (!h->have_result) {
        return fail(h, PSR_INVALID_INPUT, "no reconstruction yet");
    }
    const Workspace& ws = h->ws;
    const Counters& c = slot >= 0 ? h->cnt_host_all[slot] : h->host_cnt;
    const int D = ws.depth;
    const size_t M = (size_t)c.n_nodes, N = (size_t)c.n_points, MD = (size_t)c.level_count[D];
    struct Item { const void* p; size_t bytes; size_t stride_bytes; int rows; };
    std::vector<Item> items;
    auto one = [&](const void* p, size_t b) { items.push_back({p, b, 0, 1}); };
    auto rows = [&](const void* p, int r, size_t row_bytes, size_t stride_bytes) { items.push_back({p, row_bytes, stride_bytes, r}); };
    const size_t S = (size_t)ws.cap.nodes;
    if (nm == "px") one(ws.px, 4 * N);
    else if (nm == "py") one(ws.py, 4 * N);
    else if (nm == "pz") one(ws.pz, 4 * N);
    else if (nm == "nx") one(ws.nx, 4 * N);
    else if (nm == "ny") one(ws.ny, 4 * N);
    else if (nm == "nz") one(ws.nz, 4 * N);
    else if (nm == "point2node") one(ws.point2node, 4 * N);
    else if (nm == "key") one(ws.key, 4 * M);
    else if (nm == "pidx") one(ws.pidx, 4 * M);
    else if (nm == "pnum") one(ws.pnum, 4 * M);
    else if (nm == "parent") one(ws.parent, 4 * M);
    else if (nm == "first_child") one(ws.first_child, 4 * M);
    else if (nm == "didx") one(ws.didx, 4 * M);
    else if (nm == "dnum") one(ws.dnum, 4 * M);
    else if (nm == "depth") one(ws.ndepth, 4 * M);
    else if (nm == "enc") one(ws.enc, 4 * M);
    else if (nm == "ctr_x") one(ws.ctr_x, 4 * M);
    else if (nm == "ctr_y") one(ws.ctr_y, 4 * M);
    else if (nm == "ctr_z") one(ws.ctr_z, 4 * M);
    else if (nm == "neigh") rows(ws.neigh, 27, 4 * M, 4 * S);
    else if (nm == "node_vtx") rows(ws.node_vtx, 8, 4 * M, 4 * S);
    else if (nm == "node_edge") rows(ws.node_edge, 12, 4 * M, 4 * S);
    else if (nm == "node_face") rows(ws.node_face, 6, 4 * M, 4 * S);
    else if (nm == "vfield") rows(ws.vfield, 3, 4 * MD, 4 * (size_t)ws.cap.dnodes);
    else if (nm == "divg") one(ws.divg, 4 * M);
    else if (nm == "x") one(ws.xsol, 4 * M);
    else if (nm == "point_val") one(ws.point_val, 4 * N);
    else if (nm == "v_x") one(ws.v_x, 4 * (size_t)c.n_vertices);
    else if (nm == "v_y") one(ws.v_y, 4 * (size_t)c.n_vertices);
    else if (nm == "v_z") one(ws.v_z, 4 * (size_t)c.n_vertices);
    else if (nm == "v_owner") one(ws.v_owner, 4 * (size_t)c.n_vertices);
    else if (nm == "v_kind") one(ws.v_kind, 4 * (size_t)c.n_vertices);
    else if (nm == "v_depth") one(ws.v_depth, 4 * (size_t)c.n_vertices);
    else if (nm == "vvalue") one(ws.vvalue, 4 * (size_t)c.n_vertices);
    else if (nm == "e_owner") one(ws.e_owner, 4 * (size_t)c.n_edges);
    else if (nm == "e_kind") one(ws.e_kind, 4 * (size_t)c.n_edges);
    else if (nm == "f_owner") one(ws.f_owner, 4 * (size_t)c.n_faces);
    else if (nm == "f_kind") one(ws.f_kind, 4 * (size_t)c.n_faces);
    else if (nm == "f_hasparent") one(ws.f_hasparent, 4 * (size_t)c.n_faces);
    else if (nm == "cube_class") one(ws.cube_class, 4 * MD);
    else if (nm == "sub_root") one(ws.sub_root, 4 * (size_t)c.n_subroots);
    else if (nm == "mesh_v") one(ws.mesh_v, 12 * (size_t)c.n_mesh_vertices);
    else if (nm == "mesh_t") one(ws.mesh_t, 12 * (size_t)c.n_mesh_triangles);
    else if (nm == "mesh_c") one(ws.mesh_c, 12 * (size_t)c.n_mesh_vertices);
    else if (nm == "mesh_n") one(ws.mesh_n, 12 * (size_t)c.n_mesh_vertices);
    else if (nm == "sv_value") one(ws.sv_value, 4 * (size_t)c.n_sub_vertices);
    else if (nm == "s_cube_class") one(ws.s_cube_class, 4 * (size_t)c.n_sub_dnodes);
    else if (nm == "sub_live_vnode") one(ws.lv_vnode, 4 * (size_t)c.n_sub_dnodes);
    else if (nm == "bbox") {   // the normalisation of the last run: center[3], max edge (4 floats)
        const float v[4] = {c.center[0], c.center[1], c.center[2], c.max_edge};
        if (bytes) *bytes = sizeof(v);
        if (dst && dst_bytes >= sizeof(v)) memcpy(dst, v, sizeof(v));
        return PSR_OK;
    }
    else if (nm == "counters") { if (bytes) *bytes = sizeof(Counters); if (dst && dst_bytes >= sizeof(Counters)) memcpy(dst, &c, sizeof(Counters)); return PSR_OK; }
    else return fail(h, PSR_INVALID_INPUT, "unknown array name");
    size_t total = 0;
    for (auto& it : items) total += it.bytes * it.rows;
    if (bytes) *bytes = total;
    if (!dst) return PSR_OK;
    if (dst_bytes < total) return fail(h, PSR_OUT_OF_CAPACITY, "destination too small");
    char* d = (char*)dst;
    cudaError_t e = cudaSuccess;
    for (auto& it : items)
        for (int r = 0; r < it.rows && e == cudaSuccess; ++r) {
            e = cudaMemcpy(d, slot_ptr((const char*)it.p, slot < 0 ? 0 : slot) + r * it.stride_bytes, it.bytes,
                           cudaMemcpyDeviceToHost);
            d += it.bytes;
        }
    if (e != cudaSuccess) return cuda_fail(h, e, "debug copy");
    return PSR_OK;
}

}  // extern "C"
