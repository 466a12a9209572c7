// kg_api.cu -- the C-ABI of libkitgpu.so (include/kitgpu.h).
#include <limits>
#include <cuda_runtime.h>
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <iterator>
#include <string>
#include <vector>
#include "kg_device.cuh"
#include "kg_devflat.h"

namespace kg {
template <int D, int NDF, typename T> struct Launch {
    static cudaError_t slope(const Dev&, int, int, cudaStream_t);
    static cudaError_t solid(const Dev&, int, cudaStream_t);
    static cudaError_t wall(const Dev&, int, int, cudaStream_t);
    static cudaError_t wall_rows(const Dev&, int, double*, cudaStream_t);
    static cudaError_t flux_persistent(const Dev&, int, int, int, int*, const int32_t*, cudaStream_t);
    static cudaError_t flux_list(const Dev&, const int32_t*, int, int, cudaStream_t);
    static cudaError_t flux_reg_list(const Dev&, const int32_t*, int, int, cudaStream_t, bool = false);
    static cudaError_t flux_r2_list(const Dev&, const int32_t*, int, int, cudaStream_t);
    static cudaError_t flux_inner_list(const Dev&, const int32_t*, int, int, bool, cudaStream_t, bool);
    static int flux_occupancy(const Dev&, int);
    static cudaError_t cip(const Dev&, int, cudaStream_t);
    static cudaError_t conserve(const Dev&, const int32_t*, int, cudaStream_t);
    static cudaError_t macro_slope(const Dev&, int, int, int, double*, cudaStream_t);
    static cudaError_t criterion(const Dev&, int, int, int, const double*, double, double*, double*, cudaStream_t);
    static cudaError_t adapt(const Dev&, int, const AdaptRec*, const void*, const void*, const double*, const double*,
                             const double*, const int32_t*, const int8_t*, cudaStream_t);
    static cudaError_t vs_resolution(const Dev&, int, int, double*, cudaStream_t);
    static cudaError_t vs_flags(const Dev&, int, int, const VsFlagArgs&, cudaStream_t);
};
cudaError_t launch_residual(const Dev&, const int32_t*, int, double*, cudaStream_t);
cudaError_t launch_packed_inner_ok(const Dev&, int, uint8_t*, cudaStream_t);
}  // namespace kg

using namespace kg;

namespace kg {
// message for kg_last_error(NULL, ...) from entry points that take no handle
void set_global_error(const std::string& msg);
}

namespace {

thread_local std::string g_create_err;

// ---- small kernels: conversions, wall initialisation, step counter --------------------
template <typename T>
__global__ void to_storage(const double* __restrict__ src, T* __restrict__ dst, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) dst[i] = (T)src[i];
}
template <typename T>
__global__ void from_storage(const T* __restrict__ src, double* __restrict__ dst, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) dst[i] = (double)src[i];
}
// Block copies within one array, one CTA per (src, dst, length) triple (in elements); the
// destination blocks never overlap a source block (SolidNeighbor f <- its donor's f).
template <typename T>
__global__ void copy_blocks(T* f, const int64_t* tri) {
    const int64_t* t = tri + 3 * (int64_t)blockIdx.x;
    const int64_t src = t[0], dst = t[1], len = t[2];
    for (int64_t i = threadIdx.x; i < len; i += blockDim.x) f[dst + i] = f[src + i];
}
// The checkpoint layout of save_for_restart (IO/Restart.jl:100-117): column k of the
// nv_total x ndf matrix vs_df stacks VsData.df[:, k] of every cell in cell order.  foff:
// the cells' f offsets (ndf * nv blocks, k-major), so a cell's first row is foff[c] / ndf.
template <typename T>
__global__ void restart_gather(const T* __restrict__ f, const int64_t* __restrict__ foff, int ncell, int ndf,
                               int64_t nv_total, double* __restrict__ out) {
    for (int c = blockIdx.x; c < ncell; c += gridDim.x) {
        const int64_t o = foff[c], nv = (foff[c + 1] - o) / ndf, r0 = o / ndf;
        for (int k = 0; k < ndf; ++k)
            for (int64_t i = threadIdx.x; i < nv; i += blockDim.x) out[k * nv_total + r0 + i] = (double)f[o + k * nv + i];
    }
}
template <typename T>
__global__ void restart_scatter(const double* __restrict__ in, const int64_t* __restrict__ foff, int ncell, int ndf,
                                int64_t nv_total, T* __restrict__ f) {
    for (int c = blockIdx.x; c < ncell; c += gridDim.x) {
        const int64_t o = foff[c], nv = (foff[c + 1] - o) / ndf, r0 = o / ndf;
        for (int k = 0; k < ndf; ++k)
            for (int64_t i = threadIdx.x; i < nv; i += blockDim.x) f[o + k * nv + i] = (T)in[k * nv_total + r0 + i];
    }
}
// prim = get_prim(w) of data items [0, n) (rows of MAXW), as restart() builds its PsData
template <int D>
__global__ void prim_of_w(const double* __restrict__ w, double* __restrict__ prim, int n, double gamma) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < n) get_prim<D>(w + (int64_t)c * MAXW, gamma, prim + (int64_t)c * MAXW);
}
// Rows between the caller's packed layout (n_src rows of sw doubles) and the library's padded
// one (n_dst rows of dw >= sw doubles); padding and the rows past n_src (wall data items) are
// zero.  rows_pack is the inverse for the first n rows.
__global__ void rows_unpack(const double* __restrict__ src, int sw, int n_src, double* __restrict__ dst, int dw, int n_dst) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= (int64_t)n_dst * dw) return;
    const int64_t c = i / dw;
    const int e = (int)(i - c * dw);
    dst[i] = (c < n_src && e < sw) ? src[c * sw + e] : 0.0;
}
__global__ void rows_pack(const double* __restrict__ src, int sw, double* __restrict__ dst, int dw, int n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= (int64_t)n * dw) return;
    const int64_t c = i / dw;
    dst[i] = src[c * sw + (i - c * dw)];
}
__global__ void set_step_counter(int64_t* p, int64_t v) { *p = v; }
}  // namespace

void kg::set_global_error(const std::string& msg) { g_create_err = msg; }

namespace {

// first-fit allocator of contiguous ranges (f elements or data slots) within a pool
struct RangeAlloc {
    std::map<int64_t, int64_t> free_;   // start -> length
    int64_t cap = 0;
    void reset(int64_t c) { free_.clear(); cap = c; if (c > 0) free_[0] = c; }
    bool alloc(int64_t n, int64_t* at) {
        if (n <= 0) { *at = 0; return true; }
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= n) {
                *at = it->first;
                int64_t rest = it->second - n, ns = it->first + n;
                free_.erase(it);
                if (rest > 0) free_[ns] = rest;
                return true;
            }
        }
        return false;
    }
    void release(int64_t at, int64_t n) {
        if (n <= 0) return;
        auto it = free_.emplace(at, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) { it->second += nx->second; free_.erase(nx); }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) { pv->second += it->second; free_.erase(it); }
        }
    }
    int64_t free_total() const { int64_t t = 0; for (auto& kv : free_) t += kv.second; return t; }
};

struct Problem {
    bool live = false;
    Flat F;
    DevLayout dl;                  // F.devlay: the step arrays built on the device
    int64_t fbase = 0, fsize = 0;
    int64_t dbase = 0, dsize = 0;
    ProbParams pp{};
};

}  // namespace

struct kg_handle {
    kg_params prm{};
    int device = 0;
    cudaStream_t stream = nullptr;
    // a step's immersed-boundary kernels run on `aux` beside the flux of the fluid cells that
    // read none of their output (fork / join through the two events)
    cudaStream_t aux = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    const int32_t* d_reg = nullptr;    // fluid-list entries of regular cells (regular-cell kernel)
    const int32_t* d_nonreg = nullptr; // every other entry
    const int32_t* d_r2 = nullptr;     // regular cells whose slopes the packed kernel computes
    const int32_t* d_inner = nullptr;  // cells of the packed kernel's INNER form (2D mixed form)
    const int32_t* d_innerp = nullptr; // the same with a neighbour on another velocity grid
    int n_reg = 0, n_nonreg = 0, n_r2 = 0, n_inner = 0, n_innerp = 0;
    int64_t ph_reg = 0, ph_nonreg = 0, ph_r2 = 0, ph_inner = 0, ph_innerp = 0;   // their phase cells (profile units)
    std::string err;
    bool is_batch = false;
    bool have_state = false;       // single-problem API: state uploaded
    std::vector<Problem> probs;    // slots
    RangeAlloc fslab, dslab;
    int64_t fcap = 0, dcap = 0;
    // pools (persist across membership changes)
    std::vector<void*> pool_allocs;
    void* fA = nullptr;
    void* fB = nullptr;
    void* sdf = nullptr;
    double *w = nullptr, *prim = nullptr, *qf = nullptr, *staging = nullptr;
    ProbParams* d_probs = nullptr;
    int64_t* d_step = nullptr;
    int* d_status = nullptr;
    double* res_out = nullptr;     // [MAX_SLOTS][RES_STRIDE]
    double* h_res = nullptr;       // pinned copy
    int* h_status = nullptr;       // pinned copy
    int64_t pool_bytes = 0;
    // merged topology (rebuilt when membership changes)
    bool dirty = true;
    // the slopes of R2 cells in the packed regular-cell kernel (kg_fuse_slopes; off by default:
    // it moves less DRAM traffic but takes longer on GB300, the flux kernel being issue- and
    // latency-bound rather than bandwidth-bound)
    bool fuse_off = true;
    // the sdf of the lazy pass cells is the last step's only after enqueue_lazy_slopes ran on
    // the f that step read (set by every step of a layout with lazy items)
    bool sdf_partial = false;
    int64_t version = 0;
    std::vector<void*> topo_allocs;
    int64_t topo_bytes = 0;
    // the read-only topology arrays of a layout in one allocation
    char* arena = nullptr;
    size_t arena_cap = 0, arena_used = 0;
    char* upin = nullptr;          // pinned staging of the arena's upload
    size_t upin_cap = 0;
    bool arena_measure = false;    // first pass: only sum the sizes
    Flat M;
    Flat spare;                    // a previous problem's arrays, reused by the next flattening
    Dev dev{};
    std::vector<int32_t> live;
    int32_t* d_live = nullptr;
    int parity = 0;                // 0: f_in = fA
    // profiling
    bool prof = false;
    std::vector<std::string> pnames;
    std::vector<double> pms;
    std::vector<int64_t> pcount;
    std::vector<int64_t> punits;   // phase cells the entry's launches processed (flux kernels)
    std::vector<const char*> pname_ptrs;
    // flux schedule (autotuned): 0 one CTA per cell, 1 persistent in cell order,
    // 2 persistent with the largest velocity grids first
    int sched = 0;
    int sched_ctas = 0;           // resident CTAs per SM of the persistent grid
    bool autotune = false;
    int64_t tuned_version = -1;
    double tune_ms[8] = {0};
    int* d_counter = nullptr;
    const int32_t* d_order = nullptr;
    int64_t* d_tri = nullptr;      // wall-initialisation copies of an upload (grown on demand)
    int64_t tri_cap = 0;
    // pipelined serving (kg_serve): two copy streams and FP64 staging, made on first use
    cudaStream_t s_in = nullptr, s_out = nullptr;
    double* sv_buf = nullptr;
    int64_t sv_cap = 0;            // doubles
    // graph
    bool use_graph = false;
    cudaGraphExec_t gexec = nullptr;
    int g_nsteps = -1, g_parity = -1;
    int64_t g_version = -1;
    int64_t last_launches = 0;
    // single-problem handles build the gather form after a topology upload or an adaptation on
    // the device (kg_devflat.cu); kg_device_flatten(h, 0) selects the host builder
    bool devflat = true;
    DevScratch dscratch;
    DevLayout mdl;                 // the merged device-built layout of a batch
    DevLayout* cur_dl = nullptr;   // the device-built arrays of the current layout, if any
    // a single handle's previous pools, kept after an adaptation moved the state out of them:
    // the next adaptation that fits takes them instead of allocating (and freeing) pools
    struct PoolSet {
        std::vector<void*> allocs;
        void *fA = nullptr, *fB = nullptr, *sdf = nullptr;
        double *w = nullptr, *prim = nullptr, *qf = nullptr, *staging = nullptr;
        ProbParams* d_probs = nullptr;
        int64_t* d_step = nullptr;
        int* d_status = nullptr;
        double* res_out = nullptr;
        int* d_counter = nullptr;
        int64_t fcap = 0, dcap = 0, bytes = 0;
    } spare_pools;
};

namespace {

int fail(kg_handle* h, int code, const std::string& msg) {
    if (h) h->err = msg;
    return code;
}
int cuda_fail(kg_handle* h, cudaError_t e, const char* what) {
    return fail(h, KG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define KG_CUDA(h, call)                                              \
    do {                                                              \
        cudaError_t e__ = (call);                                     \
        if (e__ != cudaSuccess) return cuda_fail((h), e__, #call);    \
    } while (0)

size_t storage_size(const kg_handle* h) { return h->prm.precision == KG_PREC_FP64 ? sizeof(double) : sizeof(float); }

// The read-only arrays of a layout go into one device arena in two passes: the first only sums
// their sizes; the second copies each into a pinned staging block at its arena offset, and the
// block goes to the device in one copy (upload_arena).
template <typename V>
int upload_vec(kg_handle* h, const std::vector<V>& v, const V** out) {
    size_t n = std::max<size_t>(v.size(), 1) * sizeof(V);
    const size_t n256 = (n + 255) / 256 * 256;
    if (h->arena_measure) { h->arena_used += n256; *out = nullptr; return KG_OK; }
    if (!h->arena || h->arena_used + n256 > h->arena_cap || h->upin_cap < h->arena_cap)
        return fail(h, KG_ERR_ARG, "topology arena sized wrongly");
    if (!v.empty()) std::memcpy(h->upin + h->arena_used, v.data(), v.size() * sizeof(V));
    *out = (const V*)(h->arena + h->arena_used);
    h->arena_used += n256;
    return KG_OK;
}
// n bytes of the arena that a kernel fills (no upload)
int arena_reserve(kg_handle* h, size_t n, void** out) {
    const size_t n256 = (std::max<size_t>(n, 1) + 255) / 256 * 256;
    if (h->arena_measure) { h->arena_used += n256; *out = nullptr; return KG_OK; }
    if (!h->arena || h->arena_used + n256 > h->arena_cap) return fail(h, KG_ERR_ARG, "topology arena sized wrongly");
    *out = h->arena + h->arena_used;
    h->arena_used += n256;
    return KG_OK;
}
// after the measuring pass: an arena (and pinned staging) of at least arena_used bytes, kept
// from the last layout when large enough
int size_arena(kg_handle* h) {
    const size_t need = std::max<size_t>(h->arena_used, 256);
    if (h->arena_cap < need) {
        if (h->arena) cudaFree(h->arena);
        h->arena = nullptr;
        h->topo_bytes -= (int64_t)h->arena_cap;
        h->arena_cap = 0;
        const size_t cap = need + need / 8;
        void* a = nullptr;
        if (cudaMalloc(&a, cap) != cudaSuccess) return fail(h, KG_ERR_NOMEM, "cudaMalloc topology");
        h->arena = (char*)a;
        h->arena_cap = cap;
        h->topo_bytes += (int64_t)cap;
    }
    if (h->upin_cap < h->arena_cap) {
        if (h->upin) cudaFreeHost(h->upin);
        h->upin = nullptr;
        h->upin_cap = 0;
        void* p = nullptr;
        if (cudaMallocHost(&p, h->arena_cap) != cudaSuccess) return fail(h, KG_ERR_NOMEM, "cudaMallocHost topology staging");
        h->upin = (char*)p;
        h->upin_cap = h->arena_cap;
    }
    h->arena_used = 0;
    return KG_OK;
}
int upload_arena(kg_handle* h) {
    KG_CUDA(h, cudaMemcpyAsync(h->arena, h->upin, h->arena_used, cudaMemcpyHostToDevice, h->stream));
    return KG_OK;
}
int pool_alloc(kg_handle* h, size_t n, void** out) {
    void* p = nullptr;
    // 256 bytes past the end: the kernels' L2 prefetches round a block's end up to 16 bytes
    const size_t bytes = n + 256;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) return fail(h, KG_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    e = cudaMemsetAsync(p, 0, bytes, h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaMemsetAsync");
    h->pool_allocs.push_back(p);
    h->pool_bytes += (int64_t)n;
    *out = p;
    return KG_OK;
}

// keep_arena: the next layout reuses the arena (and its staging) when large enough
void free_topology(kg_handle* h, bool keep_arena = false) {
    if (h->gexec) { cudaGraphExecDestroy(h->gexec); h->gexec = nullptr; }
    h->g_nsteps = -1;
    for (void* p : h->topo_allocs) cudaFree(p);
    h->topo_allocs.clear();
    h->arena_used = 0;
    if (keep_arena) return;
    if (h->arena) cudaFree(h->arena);
    if (h->upin) cudaFreeHost(h->upin);
    h->arena = nullptr;
    h->upin = nullptr;
    h->arena_cap = h->upin_cap = 0;
    h->topo_bytes = 0;
}

// keep_arena: new pools follow at once (make_pools, adopt_pools), so the topology arena and its
// staging stay for the next layout
void free_pools(kg_handle* h, bool keep_arena = false) {
    free_topology(h, keep_arena);
    for (void* p : h->pool_allocs) cudaFree(p);
    h->pool_allocs.clear();
    h->pool_bytes = 0;
    h->fA = h->fB = h->sdf = nullptr;
    h->w = h->prim = h->qf = h->staging = nullptr;
    if (keep_arena && h->probs.size() == (size_t)MAX_SLOTS) {
        // the slot table stays: only the slots in use are emptied
        for (Problem& pb : h->probs)
            if (pb.live || pb.fsize || pb.dsize || pb.F.n_data) pb = Problem();
    } else {
        h->probs.clear();
    }
    h->live.clear();
    h->dirty = true;
    h->have_state = false;
}

// Pools for fcap f elements and dcap data slots.
int make_pools(kg_handle* h, int64_t fcap, int64_t dcap) {
    free_pools(h, true);
    const int D = h->prm.dim;
    size_t ss = storage_size(h);
    void* p;
    int rc;
    if ((rc = pool_alloc(h, fcap * ss, &h->fA))) return rc;
    if ((rc = pool_alloc(h, fcap * ss, &h->fB))) return rc;
    if ((rc = pool_alloc(h, fcap * D * ss, &h->sdf))) return rc;
    if ((rc = pool_alloc(h, sizeof(double) * dcap * MAXW, &p))) return rc; h->w = (double*)p;
    if ((rc = pool_alloc(h, sizeof(double) * dcap * MAXW, &p))) return rc; h->prim = (double*)p;
    if ((rc = pool_alloc(h, sizeof(double) * dcap * MAXD, &p))) return rc; h->qf = (double*)p;
    if (h->prm.precision != KG_PREC_FP64) { if ((rc = pool_alloc(h, sizeof(double) * fcap, &p))) return rc; h->staging = (double*)p; }
    if ((rc = pool_alloc(h, sizeof(ProbParams) * MAX_SLOTS, &p))) return rc; h->d_probs = (ProbParams*)p;
    if ((rc = pool_alloc(h, sizeof(int64_t) * MAX_SLOTS, &p))) return rc; h->d_step = (int64_t*)p;
    if ((rc = pool_alloc(h, sizeof(int) * MAX_SLOTS, &p))) return rc; h->d_status = (int*)p;
    if ((rc = pool_alloc(h, sizeof(double) * MAX_SLOTS * RES_STRIDE, &p))) return rc; h->res_out = (double*)p;
    if ((rc = pool_alloc(h, sizeof(int) * 4, &p))) return rc; h->d_counter = (int*)p;
    h->fcap = fcap; h->dcap = dcap;
    h->fslab.reset(fcap);
    h->dslab.reset(dcap);
    if (h->probs.size() != (size_t)MAX_SLOTS) h->probs.assign(MAX_SLOTS, Problem());
    h->parity = 0;
    h->dirty = true;
    // the zero fill of a pool of hundreds of GB runs for tens of ms; finish it before any
    // state upload lands in the pools
    KG_CUDA(h, cudaStreamSynchronize(h->stream));
    return KG_OK;
}

// the handle's current pools as a set, and a set adopted as the current pools (no allocation,
// no fill: an adaptation writes every data item of the new mesh before a step reads it)
kg_handle::PoolSet take_pools(kg_handle* h) {
    kg_handle::PoolSet ps;
    ps.allocs.swap(h->pool_allocs);
    ps.fA = h->fA; ps.fB = h->fB; ps.sdf = h->sdf;
    ps.w = h->w; ps.prim = h->prim; ps.qf = h->qf; ps.staging = h->staging;
    ps.d_probs = h->d_probs; ps.d_step = h->d_step; ps.d_status = h->d_status; ps.res_out = h->res_out;
    ps.d_counter = h->d_counter;
    ps.fcap = h->fcap; ps.dcap = h->dcap; ps.bytes = h->pool_bytes;
    h->fA = h->fB = h->sdf = nullptr;
    h->w = h->prim = h->qf = h->staging = nullptr;
    h->pool_bytes = 0;
    return ps;
}
int adopt_pools(kg_handle* h, kg_handle::PoolSet& ps) {
    free_pools(h, true);
    h->pool_allocs.swap(ps.allocs);
    h->fA = ps.fA; h->fB = ps.fB; h->sdf = ps.sdf;
    h->w = ps.w; h->prim = ps.prim; h->qf = ps.qf; h->staging = ps.staging;
    h->d_probs = ps.d_probs; h->d_step = ps.d_step; h->d_status = ps.d_status; h->res_out = ps.res_out;
    h->d_counter = ps.d_counter;
    h->pool_bytes = ps.bytes;
    h->fcap = ps.fcap; h->dcap = ps.dcap;
    ps = kg_handle::PoolSet();
    h->fslab.reset(h->fcap);
    h->dslab.reset(h->dcap);
    if (h->probs.size() != (size_t)MAX_SLOTS) h->probs.assign(MAX_SLOTS, Problem());
    h->parity = 0;
    h->dirty = true;
    KG_CUDA(h, cudaMemsetAsync(h->d_status, 0, sizeof(int) * MAX_SLOTS, h->stream));
    KG_CUDA(h, cudaMemsetAsync(h->d_step, 0, sizeof(int64_t) * MAX_SLOTS, h->stream));
    return KG_OK;
}
void release_pools(kg_handle::PoolSet& ps) {
    for (void* p : ps.allocs) cudaFree(p);
    ps = kg_handle::PoolSet();
}

int prof_slot(kg_handle* h, const char* name) {
    for (size_t i = 0; i < h->pnames.size(); ++i)
        if (h->pnames[i] == name) return (int)i;
    h->pnames.push_back(name);
    h->pms.push_back(0.0);
    h->pcount.push_back(0);
    h->punits.push_back(0);
    return (int)h->pnames.size() - 1;
}

// Dispatch on (dim, storage) for the templated launchers.
template <typename Fn>
cudaError_t dispatch(const kg_handle* h, Fn fn) {
    if (h->prm.dim == 2) {
        if (h->prm.precision == KG_PREC_FP64) return fn(Launch<2, 2, double>());
        return fn(Launch<2, 2, float>());
    }
    if (h->prm.precision == KG_PREC_FP64) return fn(Launch<3, 1, double>());
    return fn(Launch<3, 1, float>());
}

ProbParams params_of(const kg_params& p, double dt) {
    ProbParams pp{};
    pp.gamma = p.gamma; pp.K = p.K; pp.Pr = p.Pr; pp.omega = p.omega; pp.mu_ref = p.mu_ref;
    pp.dt = dt; pp.check = p.st_check_interval;
    pp.dtf = (float)dt; pp.Kf = (float)p.K; pp.mu2f = (float)(2.0 * p.mu_ref);
    pp.omf = (float)(1.0 - p.omega); pp.shkf = (float)(0.8 * (1.0 - p.Pr));
    return pp;
}

// new dt of a problem, on the device too when the merged table is current
int set_prob_dt(kg_handle* h, int slot, double dt) {
    ProbParams& pp = h->probs[slot].pp;
    pp.dt = dt;
    pp.dtf = (float)dt;
    if (!h->dirty) KG_CUDA(h, cudaMemcpyAsync(&h->d_probs[slot], &pp, sizeof(ProbParams), cudaMemcpyHostToDevice, h->stream));
    KG_CUDA(h, cudaStreamSynchronize(h->stream));   // pp is host memory the copy reads
    return KG_OK;
}

// Host wall time of the phases of a call, into the profile table when profiling is on.
struct PhaseClock {
    kg_handle* h;
    std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
    void mark(const char* name) {
        if (!h->prof) return;
        const auto n = std::chrono::steady_clock::now();
        const int k = prof_slot(h, name);
        h->pms[k] += std::chrono::duration<double, std::milli>(n - t).count();
        h->pcount[k] += 1;
        t = n;
    }
};

// The gather form of a problem: on the device (kg_devflat.cu) unless the host builder was
// selected.
int build_layout(kg_handle* h, const kg_topology& topo, int slot, Flat& F, DevLayout& dl, std::string& err) {
    if (!h->devflat) return flatten(h->prm, topo, F, err);
    double t[4] = {0, 0, 0, 0};
    const int rc = device_flatten(h->prm, topo, slot, h->stream, F, dl, h->dscratch, err, t);
    if (h->prof) {
        const char* names[4] = {"flatten:host", "flatten:upload", "flatten:count", "flatten:build"};
        for (int k = 0; k < 4; ++k) {
            const int e = prof_slot(h, names[k]);
            h->pms[e] += t[k];
            h->pcount[e] += 1;
        }
    }
    return rc;
}

// Rebuilds the merged gather form of the live problems and uploads it.
int rebuild(kg_handle* h) {
    if (!h->dirty) return KG_OK;
    PhaseClock clk{h};
    cudaStreamSynchronize(h->stream);
    free_topology(h, true);
    std::vector<Part> parts;
    h->live.clear();
    for (int s = 0; s < (int)h->probs.size(); ++s) {
        Problem& pb = h->probs[s];
        if (!pb.live) continue;
        parts.push_back(Part{&pb.F, pb.fbase, (int32_t)pb.dbase, s});
        h->live.push_back(s);
    }
    std::vector<int32_t> ranges;
    const bool fuse = !h->fuse_off && h->prm.dim == 2 && h->prm.precision == KG_PREC_MIXED && h->prm.marching != KG_MARCH_CIP;
    // problems whose step arrays were built on the device: the host-side arrays are merged here;
    // a single problem at data and f base 0 keeps its own device arrays, several are merged on
    // the device (device_merge); then the R2 records on the device and the slope work items
    bool all_dev = !parts.empty();
    for (const Part& p : parts) all_dev = all_dev && p.F->devlay;
    DevLayout* DL = nullptr;
    if (all_dev)
        DL = (parts.size() == 1 && parts[0].dbase == 0 && parts[0].fbase == 0) ? &h->probs[parts[0].slot].dl : &h->mdl;
    merge(parts, (int32_t)h->dcap, h->M, ranges, fuse, DL != nullptr);
    Flat& M = h->M;
    h->cur_dl = DL;
    if (DL == &h->mdl) {
        // each part's offsets as merge() accumulates them, and the merged start of its passes
        size_t npass = 0;
        for (const Part& p : parts) npass = std::max(npass, p.F->pass_cells_off.size() - 1);
        std::vector<MergeIn> mi(parts.size());
        int32_t run = 0;
        for (size_t ps = 0; ps < npass; ++ps)
            for (size_t q = 0; q < parts.size(); ++q) {
                const Flat& F = *parts[q].F;
                if (ps + 1 >= F.pass_cells_off.size()) continue;
                mi[q].pass_base.push_back(run);
                run += F.pass_cells_off[ps + 1] - F.pass_cells_off[ps];
            }
        int32_t snb = 0, sops = 0, cacc = 0, incacc = 0, bcacc = 0, pairacc = 0, Gacc = 0;
        int64_t PGacc = 0;
        for (size_t q = 0; q < parts.size(); ++q) {
            const Flat& F = *parts[q].F;
            const DevLayout& L = h->probs[parts[q].slot].dl;
            MergeIn& m = mi[q];
            m.L = &L;
            m.fbase = parts[q].fbase; m.dbase = parts[q].dbase;
            m.snb = snb; m.sops = sops; m.cacc = cacc; m.incacc = incacc; m.bcacc = bcacc; m.pairacc = pairacc;
            m.Gacc = Gacc; m.PGacc = PGacc;
            m.pass_off = F.pass_cells_off;
            snb += (int32_t)L.n_slope_nbr; sops += (int32_t)L.n_slope_ops; cacc += (int32_t)L.n_crit_nbr;
            incacc += (int32_t)L.n_inc; bcacc += (int32_t)L.n_bc; pairacc += (int32_t)F.p_off.size() - 1;
            Gacc += (int32_t)F.g_off.size() - 1; PGacc += (int64_t)F.vw.size();
        }
        std::string err;
        const int rc = device_merge(mi, h->dcap, (int64_t)M.pass_cells.size(), M.foff.data(), M.dnv.data(), M.dim,
                                    h->stream, h->mdl, h->dscratch, err);
        if (rc) return fail(h, rc, err);
    }
    clk.mark("rebuild:merge");
    if (DL) {
        std::string err;
        const int rc = device_r2(M, *DL, fuse, h->stream, M.fluid_r2, err);
        if (rc) return fail(h, rc, err);
        slope_items(M, (int32_t)h->dcap, fuse);
    }
    clk.mark("rebuild:r2");
    if (!parts.empty()) {
        if (M.max_inc > MAX_INC) return fail(h, KG_ERR_TOPOLOGY, "a cell has more face incidences than supported");
        int dev_smem = 0;
        cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device);
        // dynamic shared memory of the flux and wall kernels plus a reserve for their static arrays
        const size_t sa = storage_size(h);
        // the flux kernel's convected f can move to global memory; its tables and the wall
        // kernel's cannot
        const size_t sflux = (size_t)std::max(2, M.max_bcm) * M.dim * M.max_axis * sa + 16384;
        const size_t swall = (size_t)M.dim * M.max_axis * sa + M.max_nv + 4096;
        const size_t smax = std::max(sflux, swall);
        if (smax > (size_t)dev_smem) return fail(h, KG_ERR_TOPOLOGY, "velocity grid too large for one CTA's shared memory");
    }
    // the launch lists of the flux kernels are filled in below (their arena regions reserved)
    std::vector<int32_t> order, reg, nonreg, r2, inner, innerp;
    Dev& P = h->dev;
    P = Dev{};
    P.dim = h->prm.dim; P.ndf = h->prm.ndf; P.n_cells = M.n_cells; P.n_walls = M.n_walls;
    P.PG = (int64_t)M.vw.size();
    // the read-only arrays: sizes first, then one arena, then the copies
    uint8_t* inner_flags = nullptr;
    auto upload_all = [&]() -> int {
#define UP(field, vec) do { int r__ = upload_vec(h, M.vec, &P.field); if (r__) return r__; } while (0)
        UP(g_off, g_off); UP(vlev, vlev); UP(vw, vw); UP(vu, vu);
        UP(vuf, vuf); UP(vwf, vwf); UP(ax_off, ax_off); UP(ax_val, ax_val); UP(ax_hi, ax_hi); UP(ax_lo, ax_lo); UP(vidx, vidx);
        UP(foff, foff); UP(dgrid, dgrid); UP(dbe, dbe); UP(dmid, dmid); UP(dds, dds); UP(dinvv, dinvv); UP(dnv, dnv); UP(dprob, dprob);
        UP(p_off, p_off); UP(p_j0, p_j0); UP(p_cnt, p_cnt);
        UP(slope_items, slope_items);
        if (!DL) {
            UP(slope_ops, slope_ops); UP(pass_cells, pass_cells); UP(cell_slope_op, cell_slope_op); UP(slope_nbr, slope_nbr);
            UP(fluid_cells, fluid_cells); UP(fluid_reg, fluid_reg); UP(fcrec, fcrec); UP(regrec, regrec); UP(r2rec, r2rec); UP(screc, screc); UP(crit_ops, crit_ops); UP(crit_nbr, crit_nbr); UP(inc_off, inc_off); UP(inc, inc); UP(bc_prim, bc_prim); UP(bc_hl, bc_hl);
        }
        UP(solid_ops, solid_ops); UP(wall_ops, wall_ops); UP(ib_nbr, ib_nbr); UP(ib_dx, ib_dx);
        UP(cut_idx, cut_idx); UP(cut_gw, cut_gw); UP(cut_sw, cut_sw); UP(cvcw, cvcw);
#undef UP
        void* lr[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
        int r = KG_OK;
        for (int k = 0; k < 6 && !r; ++k) r = arena_reserve(h, sizeof(int32_t) * std::max(M.n_fluid, 1), &lr[k]);
        if (!r) r = arena_reserve(h, std::max(M.n_fluid, 1), &lr[6]);
        h->d_order = (const int32_t*)lr[0]; h->d_reg = (const int32_t*)lr[1]; h->d_nonreg = (const int32_t*)lr[2];
        h->d_r2 = (const int32_t*)lr[3]; h->d_inner = (const int32_t*)lr[4]; h->d_innerp = (const int32_t*)lr[5];
        inner_flags = (uint8_t*)lr[6];
        const int32_t* dlive = nullptr;
        if (!r) r = upload_vec(h, h->live, &dlive);
        h->d_live = const_cast<int32_t*>(dlive);
        void* cr = nullptr;
        if (!r) r = arena_reserve(h, sizeof(double) * std::max<int64_t>(M.n_fluid, 1) * 2 * MAXW, &cr);
        P.cell_res = (double*)cr;
        return r;
    };
    h->arena_measure = true;
    h->arena_used = 0;
    upload_all();
    h->arena_measure = false;
    { int r = size_arena(h); if (r) return r; }
    { int r = upload_all(); if (r) return r; }
    { int r = upload_arena(h); if (r) return r; }
    clk.mark("rebuild:upload");
    if (DL) {
        P.slope_ops = DL->slope_ops; P.pass_cells = DL->pass_cells; P.cell_slope_op = DL->cell_slope_op;
        P.slope_nbr = DL->slope_nbr; P.fluid_cells = DL->fluid_cells; P.fluid_reg = DL->fluid_reg; P.fcrec = DL->fcrec;
        P.regrec = DL->regrec; P.r2rec = DL->r2rec; P.screc = DL->screc; P.crit_ops = DL->crit_ops; P.crit_nbr = DL->crit_nbr;
        P.inc_off = DL->inc_off; P.inc = DL->inc; P.bc_prim = DL->bc_prim; P.bc_hl = DL->bc_hl;
    }
    P.max_axis = M.max_axis;
    P.max_bcm = M.max_bcm;
    {
        // explicit work items when a pass cell is split into chunks or the items are not the
        // pass cells in order (lazy items moved to the end); a chunk is SLOPE_CHUNK velocity
        // cells, or the whole cell
        bool by_size = false, in_order = (int64_t)M.slope_items.size() / 2 == (int64_t)M.pass_cells.size();
        for (int32_t m : M.pass_cells) by_size |= M.dnv[m] > 2 * SLOPE_CHUNK;
        for (size_t i = 0; in_order && i < M.slope_items.size() / 2; ++i) in_order = M.slope_items[2 * i] == (int32_t)i;
        P.slope_split = by_size || !in_order;
        P.slope_chunk = by_size ? SLOPE_CHUNK : (1 << 30);
    }
    if (M.n_fluid > 0) {
        // stage the flux kernel's convected f in global memory when shared memory would cost
        // resident CTAs (or not fit at all)
        int dev_smem = 0;
        cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device);
        const size_t sa = storage_size(h);
        const size_t full = ((size_t)M.ndf * M.max_nv + (size_t)std::max(2, M.max_bcm) * M.dim * M.max_axis) * sa + 16384;
        P.fst_global = 0;
        const int occ_smem = full <= (size_t)dev_smem
            ? (int)dispatch(h, [&](auto L) { return (cudaError_t)decltype(L)::flux_occupancy(P, M.max_nv); }) : 0;
        P.fst_global = 1;
        const int occ_glob = (int)dispatch(h, [&](auto L) { return (cudaError_t)decltype(L)::flux_occupancy(P, M.max_nv); });
        P.fst_global = occ_glob > occ_smem ? 1 : 0;
        // small velocity grids: the per-cell fixed work (setup, reductions, the scalar chain)
        // outweighs the per-velocity work, and 128-thread CTAs keep twice the cells in flight;
        // 2D layouts take 128 threads at every grid size (the packed regular-cell kernel issues
        // half the instructions per velocity cell, so the per-cell fixed work weighs more)
        const double mean_nv = (double)M.phase_cells / (double)M.n_fluid;
        P.flux_nt = (!P.fst_global && (mean_nv < 1024.0 || M.dim == 2)) ? 128 : BLOCK;
        // (3D layouts: 128 threads at every grid size -- twice the work items in flight per SM;
        // the sphere's slope passes 7.4 -> 7.0 ms per launch, while the 2D cylinder's grids of
        // 2,304 velocity cells are faster at 256)
        P.slope_nt = (mean_nv < 1024.0 || M.dim == 3) ? 128 : BLOCK;
        // the packed kernels of a layout of many cells with small velocity grids (a batch): 64
        // threads, twice the cells in flight per SM (batched workload, mean 700 velocity cells:
        // 30.5 -> 35.1 G updates/s); with few cells (the 848-cell Sod tube: 9.1 -> 8.0) each
        // cell's longer chain of passes costs more than the extra cells in flight bring
        int nsm = 0;
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, h->device);
        P.packed_nt = (mean_nv < 1024.0 && (int64_t)M.n_fluid >= (int64_t)24 * std::max(nsm, 1)) ? 64 : P.flux_nt;
    }
    {
        // the launch lists of the flux kernels: the regular fluid cells (the regular-cell kernel;
        // a regular cell never reads a solid cell or wall record) and those whose slopes the
        // packed kernel computes; in the 2D mixed form the cells of the packed kernel's INNER
        // form (inner faces to cells on their own grid only, hanging faces included); the others,
        // also largest velocity grids first (persistent schedule)
        std::vector<uint8_t> inner_ok((size_t)M.n_fluid, 0);
        const bool packed = h->prm.dim == 2 && h->prm.precision == KG_PREC_MIXED && !P.fst_global &&
                            h->prm.marching != KG_MARCH_CIP;
        if (packed && M.n_fluid > 0) {
            KG_CUDA(h, launch_packed_inner_ok(P, M.n_fluid, inner_flags, h->stream));
            KG_CUDA(h, cudaMemcpyAsync(inner_ok.data(), inner_flags, (size_t)M.n_fluid, cudaMemcpyDeviceToHost, h->stream));
            KG_CUDA(h, cudaStreamSynchronize(h->stream));
        }
        for (int q = 0; q < M.n_fluid; ++q) {
            if (!M.fluid_reg[q]) {
                if (inner_ok[q] == 1) inner.push_back(q);
                else if (inner_ok[q] == 2) innerp.push_back(q);
                else { nonreg.push_back(q); order.push_back(q); }
            } else if (M.fluid_r2[q]) r2.push_back(q);
            else reg.push_back(q);
        }
        std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) {
            return M.dnv[M.fluid_cells[x]] > M.dnv[M.fluid_cells[y]];
        });
        h->n_reg = (int)reg.size();
        h->n_nonreg = (int)nonreg.size();
        h->n_r2 = (int)r2.size();
        h->n_inner = (int)inner.size();
        h->n_innerp = (int)innerp.size();
        auto phase = [&](const std::vector<int32_t>& l) {
            int64_t n = 0;
            for (int32_t q : l) n += M.dnv[M.fluid_cells[q]];
            return n;
        };
        h->ph_reg = phase(reg);
        h->ph_nonreg = phase(nonreg);
        h->ph_r2 = phase(r2);
        h->ph_inner = phase(inner);
        h->ph_innerp = phase(innerp);
        const std::vector<int32_t>* lists[6] = {&order, &reg, &nonreg, &r2, &inner, &innerp};
        const int32_t* dst[6] = {h->d_order, h->d_reg, h->d_nonreg, h->d_r2, h->d_inner, h->d_innerp};
        for (int k = 0; k < 6; ++k)
            if (!lists[k]->empty())
                KG_CUDA(h, cudaMemcpyAsync(const_cast<int32_t*>(dst[k]), lists[k]->data(), sizeof(int32_t) * lists[k]->size(),
                                           cudaMemcpyHostToDevice, h->stream));
    }
    clk.mark("rebuild:lists");

    // per-slot parameters with the fluid ranges of this layout
    std::vector<ProbParams> table(MAX_SLOTS);
    for (size_t q = 0; q < parts.size(); ++q) {
        Problem& pb = h->probs[parts[q].slot];
        pb.pp.fluid_begin = ranges[2 * q];
        pb.pp.fluid_end = ranges[2 * q + 1];
        pb.pp.slot = parts[q].slot;
    }
    for (int s = 0; s < MAX_SLOTS; ++s) table[s] = h->probs[s].pp;
    KG_CUDA(h, cudaMemcpyAsync(h->d_probs, table.data(), sizeof(ProbParams) * MAX_SLOTS, cudaMemcpyHostToDevice, h->stream));
    KG_CUDA(h, cudaStreamSynchronize(h->stream));   // host vectors of this layout stay alive until here
    P.probs = h->d_probs;
    P.prob_step = h->d_step;
    P.status = h->d_status;
    P.w = h->w; P.prim = h->prim; P.qf = h->qf;
    P.sdf = h->sdf;
    P.flux = h->prm.flux; P.marching = h->prm.marching;
    h->dirty = false;
    h->version += 1;
    clk.mark("rebuild:params");
    return KG_OK;
}

// The flux of every fluid cell: the regular cells on their own kernel (one CTA per cell), then
// the others with one CTA per cell (schedule 0) or on persistent CTAs (1: natural order, 2:
// largest velocity grids first).
// The flux of the fluid cells by list: 0 the regular cells, 1 the R2 cells, 2 the others
// (under the schedule `sched`).
// (pdl: parts 3 and 4 launched as programmatic dependents of the packed kernel before them)
cudaError_t launch_flux_part(kg_handle* h, const Dev& P, int part, int sched, int ctas, cudaStream_t s, bool pdl) {
    const Flat& F = h->M;
    if (part == 0) return dispatch(h, [&](auto L) { return decltype(L)::flux_reg_list(P, h->d_reg, h->n_reg, F.max_nv, s); });
    if (part == 1) return dispatch(h, [&](auto L) { return decltype(L)::flux_r2_list(P, h->d_r2, h->n_r2, F.max_nv, s); });
    if (part == 3) return dispatch(h, [&](auto L) { return decltype(L)::flux_inner_list(P, h->d_inner, h->n_inner, F.max_nv, false, s, pdl); });
    if (part == 4) return dispatch(h, [&](auto L) { return decltype(L)::flux_inner_list(P, h->d_innerp, h->n_innerp, F.max_nv, true, s, pdl); });
    if (h->n_nonreg == 0) return cudaSuccess;
    if (sched == 0) return dispatch(h, [&](auto L) { return decltype(L)::flux_list(P, h->d_nonreg, h->n_nonreg, F.max_nv, s); });
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, h->device);
    int grid = std::max(1, std::min(h->n_nonreg, nsm * std::max(ctas, 1)));
    const int32_t* order = sched == 2 ? h->d_order : h->d_nonreg;
    return dispatch(h, [&](auto L) { return decltype(L)::flux_persistent(P, h->n_nonreg, F.max_nv, grid, h->d_counter, order, s); });
}

// the packed forms of a step chained by programmatic dependent launch (0: ordinary launches)
#ifndef KG_PDL
#define KG_PDL 1
#endif
cudaError_t launch_flux(kg_handle* h, const Dev& P, int sched, int ctas, cudaStream_t s) {
    cudaError_t e = cudaSuccess;
    for (int part = 0; part < 5 && e == cudaSuccess; ++part) e = launch_flux_part(h, P, part, sched, ctas, s, false);
    return e;
}

// Autotuner: times the flux schedules on the current layout and keeps the fastest.  Every
// candidate does the same per-cell arithmetic, so the choice never changes results; the
// per-cell state the trial launches touch (w, prim, qf, status) is restored afterwards.
int autotune_flux(kg_handle* h) {
    const Flat& F = h->M;
    if (F.n_fluid == 0) return KG_OK;
    Dev P = h->dev;
    P.f_in = h->parity == 0 ? h->fA : h->fB;
    P.f_out = h->parity == 0 ? h->fB : h->fA;
    int occ = dispatch(h, [&](auto L) { return (cudaError_t)decltype(L)::flux_occupancy(P, F.max_nv); });
    struct Cand { int sched, ctas; };
    std::vector<Cand> cands = {{0, 0}, {1, std::max(occ, 1)}, {2, std::max(occ, 1)}};
    if (occ > 1) cands.push_back({2, occ - 1});
    const size_t nw = sizeof(double) * h->dcap * MAXW, nq = sizeof(double) * h->dcap * MAXD;
    std::vector<char> bw(nw), bp(nw), bq(nq);
    std::vector<int> bs(MAX_SLOTS);
    KG_CUDA(h, cudaMemcpyAsync(bw.data(), h->w, nw, cudaMemcpyDeviceToHost, h->stream));
    KG_CUDA(h, cudaMemcpyAsync(bp.data(), h->prim, nw, cudaMemcpyDeviceToHost, h->stream));
    KG_CUDA(h, cudaMemcpyAsync(bq.data(), h->qf, nq, cudaMemcpyDeviceToHost, h->stream));
    KG_CUDA(h, cudaMemcpyAsync(bs.data(), h->d_status, sizeof(int) * MAX_SLOTS, cudaMemcpyDeviceToHost, h->stream));
    KG_CUDA(h, cudaStreamSynchronize(h->stream));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0); cudaEventCreate(&e1);
    double best = 1e300;
    int bi = 0;
    for (size_t c = 0; c < cands.size(); ++c) {
        cudaError_t e = launch_flux(h, P, cands[c].sched, cands[c].ctas, h->stream);   // warm-up
        if (e != cudaSuccess) return cuda_fail(h, e, "autotune");
        cudaEventRecord(e0, h->stream);
        for (int r = 0; r < 3; ++r) launch_flux(h, P, cands[c].sched, cands[c].ctas, h->stream);
        cudaEventRecord(e1, h->stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (c < 8) h->tune_ms[c] = ms / 3.0;
        if (ms < best) { best = ms; bi = (int)c; }
    }
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    KG_CUDA(h, cudaMemcpyAsync(h->w, bw.data(), nw, cudaMemcpyHostToDevice, h->stream));
    KG_CUDA(h, cudaMemcpyAsync(h->prim, bp.data(), nw, cudaMemcpyHostToDevice, h->stream));
    KG_CUDA(h, cudaMemcpyAsync(h->qf, bq.data(), nq, cudaMemcpyHostToDevice, h->stream));
    KG_CUDA(h, cudaMemcpyAsync(h->d_status, bs.data(), sizeof(int) * MAX_SLOTS, cudaMemcpyHostToDevice, h->stream));
    KG_CUDA(h, cudaStreamSynchronize(h->stream));
    h->sched = cands[bi].sched;
    h->sched_ctas = cands[bi].ctas;
    h->tuned_version = h->version;
    if (h->gexec) { cudaGraphExecDestroy(h->gexec); h->gexec = nullptr; h->g_nsteps = -1; }
    return KG_OK;
}

// One step of every live problem on the handle's stream (graph-capturable).
// The level passes of slope! on the current f (the first phase of a step).
int n_slope_passes(const Flat& F) { return std::max(0, (int)F.pass_items_off.size() - 2); }
cudaError_t enqueue_slopes(kg_handle* h, const Dev& P, cudaStream_t s) {
    const Flat& F = h->M;
    const int npass = n_slope_passes(F);
    for (int p = 0; p < npass; ++p) {
        const int base = F.pass_items_off[p], n = F.pass_items_off[p + 1] - base;
        if (n <= 0) continue;
        cudaError_t e = dispatch(h, [&](auto L) { return decltype(L)::slope(P, base, n, s); });
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}
// The lazy items: the slopes of the cells whose flux kernel computes them and whose slopes no
// other cell reads in a step (every slope of the regular form, so one launch in any order).
cudaError_t enqueue_lazy_slopes(kg_handle* h, const Dev& P, cudaStream_t s) {
    const Flat& F = h->M;
    if (F.pass_items_off.size() < 2) return cudaSuccess;
    const int base = F.pass_items_off[F.pass_items_off.size() - 2], n = F.pass_items_off.back() - base;
    if (n <= 0) return cudaSuccess;
    return dispatch(h, [&](auto L) { return decltype(L)::slope(P, base, n, s); });
}
// slope! on the current f for every pass cell (the sync points that recompute the slopes:
// the criterion, an adaptation, save_result's rows)
cudaError_t enqueue_slopes_full(kg_handle* h, const Dev& P, cudaStream_t s) {
    cudaError_t e = enqueue_slopes(h, P, s);
    if (e == cudaSuccess) e = enqueue_lazy_slopes(h, P, s);
    if (e == cudaSuccess) h->sdf_partial = false;
    return e;
}
// Before a sync point reads the slopes the last step used: the lazy cells' slopes from the f
// that step read (the other f buffer, whose fluid cells the step did not write).
bool has_lazy_slopes(const kg_handle* h) {
    const Flat& F = h->M;
    return F.pass_items_off.size() >= 2 && F.pass_items_off.back() > F.pass_items_off[F.pass_items_off.size() - 2];
}
int complete_last_slopes(kg_handle* h) {
    if (!h->sdf_partial) return KG_OK;
    Dev P = h->dev;
    P.f_in = h->parity == 0 ? h->fB : h->fA;
    KG_CUDA(h, enqueue_lazy_slopes(h, P, h->stream));
    h->sdf_partial = false;
    return KG_OK;
}

// Timed launches of a profiled step, added to the profile table when the step's work is done.
struct ProfSpans {
    kg_handle* h;
    struct Span { const char* name; int64_t units; cudaEvent_t a, b; };
    std::vector<Span> v;
    ~ProfSpans() {
        if (v.empty()) return;
        cudaEventSynchronize(v.back().b);
        for (const Span& x : v) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, x.a, x.b) == cudaSuccess) {
                const int k = prof_slot(h, x.name);
                h->pms[k] += ms;
                h->pcount[k] += 1;
                h->punits[k] += x.units;
            }
            cudaEventDestroy(x.a);
            cudaEventDestroy(x.b);
        }
    }
};

int enqueue_step(kg_handle* h, bool timed, int64_t* launches) {
    Flat& F = h->M;
    Dev P = h->dev;
    P.f_in = h->parity == 0 ? h->fA : h->fB;
    P.f_out = h->parity == 0 ? h->fB : h->fA;
    cudaStream_t s = h->stream;
    // profiling: an event pair around each launch, read once the step's last launch is done
    // (the kernels run back to back as in an unprofiled step; no host wait between them)
    ProfSpans spans{h};
    cudaEvent_t e0 = nullptr;
    auto begin = [&]() {
        if (!timed) return;
        cudaEventCreate(&e0);
        cudaEventRecord(e0, s);
    };
    auto end = [&](const char* name, int64_t units = 0) {
        if (!timed) return;
        cudaEvent_t e1 = nullptr;
        cudaEventCreate(&e1);
        cudaEventRecord(e1, s);
        spans.v.push_back({name, units, e0, e1});
    };
    cudaError_t e;
    int npass = n_slope_passes(F);
    for (int p = 0; p < npass; ++p) {
        int base = F.pass_items_off[p], n = F.pass_items_off[p + 1] - base;
        if (n <= 0) continue;
        begin();
        e = dispatch(h, [&](auto L) { return decltype(L)::slope(P, base, n, s); });
        if (e != cudaSuccess) return cuda_fail(h, e, "slope_kernel");
        end("slope_kernel");
        ++*launches;
    }
    const int n_main = (h->n_r2 > 0 ? h->n_r2 : h->n_reg) + h->n_inner + h->n_innerp;
    const int n_aux = h->n_nonreg + (h->n_r2 > 0 ? h->n_reg : 0);
    if (!timed && h->sched == 0 && n_main > 0 && n_aux > 0) {
        // two streams after the slopes: the regular cells whose slopes the flux kernel computes
        // (or, without those, the other regular cells) on the handle's stream; the IB kernels
        // and then the flux of every other cell (those that read the IB kernels' output among
        // them) on the second, higher-priority stream, whose CTAs take SM slots first as they
        // free up; the step ends on one tail
        cudaStream_t a = h->aux;
        KG_CUDA(h, cudaEventRecord(h->ev_fork, s));
        KG_CUDA(h, cudaStreamWaitEvent(a, h->ev_fork, 0));
        if (!F.solid_ops.empty()) {
            e = dispatch(h, [&](auto L) { return decltype(L)::solid(P, (int)F.solid_ops.size(), a); });
            if (e != cudaSuccess) return cuda_fail(h, e, "solid_kernel");
            ++*launches;
        }
        if (!F.wall_ops.empty()) {
            e = dispatch(h, [&](auto L) { return decltype(L)::wall(P, (int)F.wall_ops.size(), F.max_nv, a); });
            if (e != cudaSuccess) return cuda_fail(h, e, "wall_kernel");
            ++*launches;
        }
        e = dispatch(h, [&](auto L) { return decltype(L)::flux_list(P, h->d_nonreg, h->n_nonreg, F.max_nv, a); });
        if (e != cudaSuccess) return cuda_fail(h, e, "flux_collide_kernel");
        // the handle's stream: the packed forms (none reads an IB output), the costliest cells
        // first -- the paired INNER form, the INNER form, then the regular cells, whose many short
        // CTAs end the phase -- each after the first launched as a programmatic dependent of the
        // one before, so that its CTAs start on the SMs the other's last wave frees
        const bool chain = KG_PDL && h->n_r2 == 0 && h->prm.dim == 2 && h->prm.precision == KG_PREC_MIXED &&
                           !P.fst_global && h->prm.marching != KG_MARCH_CIP;
        if (h->n_r2 > 0) {
            e = dispatch(h, [&](auto L) { return decltype(L)::flux_reg_list(P, h->d_reg, h->n_reg, F.max_nv, a); });
            if (e != cudaSuccess) return cuda_fail(h, e, "flux_collide_kernel");
            e = dispatch(h, [&](auto L) { return decltype(L)::flux_r2_list(P, h->d_r2, h->n_r2, F.max_nv, s); });
            if (e != cudaSuccess) return cuda_fail(h, e, "flux_packed_kernel_r2");
            e = launch_flux_part(h, P, 3, 0, 0, s, false);
            if (e == cudaSuccess) e = launch_flux_part(h, P, 4, 0, 0, s, false);
            if (e != cudaSuccess) return cuda_fail(h, e, "flux_packed_inner_kernel");
        } else {
            bool after = false;   // a packed-form kernel launched before on this stream
            if (h->n_innerp > 0) {
                e = launch_flux_part(h, P, 4, 0, 0, s, false);
                if (e != cudaSuccess) return cuda_fail(h, e, "flux_packed_inner_kernel_paired");
                after = true;
            }
            if (h->n_inner > 0) {
                e = launch_flux_part(h, P, 3, 0, 0, s, chain && after);
                if (e != cudaSuccess) return cuda_fail(h, e, "flux_packed_inner_kernel");
                after = true;
            }
            e = dispatch(h, [&](auto L) { return decltype(L)::flux_reg_list(P, h->d_reg, h->n_reg, F.max_nv, s, chain && after); });
            if (e != cudaSuccess) return cuda_fail(h, e, "flux_packed_kernel");
        }
        KG_CUDA(h, cudaEventRecord(h->ev_join, a));
        KG_CUDA(h, cudaStreamWaitEvent(s, h->ev_join, 0));
        *launches += (h->n_nonreg > 0) + (h->n_reg > 0) + (h->n_r2 > 0) + (h->n_inner > 0) + (h->n_innerp > 0);
        if (h->prm.marching == KG_MARCH_CIP) {
            e = dispatch(h, [&](auto L) { return decltype(L)::cip(P, F.n_fluid, s); });
            if (e != cudaSuccess) return cuda_fail(h, e, "cip_kernel");
            ++*launches;
        }
        e = launch_residual(P, h->d_live, (int)h->live.size(), h->res_out, s);
        if (e != cudaSuccess) return cuda_fail(h, e, "residual_kernel");
        ++*launches;
        h->parity ^= 1;
        return KG_OK;
    }
    if (!F.solid_ops.empty()) {
        begin();
        e = dispatch(h, [&](auto L) { return decltype(L)::solid(P, (int)F.solid_ops.size(), s); });
        if (e != cudaSuccess) return cuda_fail(h, e, "solid_kernel");
        end("solid_kernel");
        ++*launches;
    }
    if (!F.wall_ops.empty()) {
        begin();
        e = dispatch(h, [&](auto L) { return decltype(L)::wall(P, (int)F.wall_ops.size(), F.max_nv, s); });
        if (e != cudaSuccess) return cuda_fail(h, e, "wall_kernel");
        end("wall_kernel");
        ++*launches;
    }
    if (F.n_fluid > 0) {
        // one timed span per flux kernel: the regular cells' kernel (the packed FP32 kernel in
        // the 2D mixed form outside CIP marching), the R2 cells' and the other cells'
        const bool packed = h->prm.dim == 2 && h->prm.precision == KG_PREC_MIXED && !P.fst_global &&
                            h->prm.marching != KG_MARCH_CIP;
        const char* names[5] = {packed ? "flux_packed_kernel" : "flux_regular_kernel", "flux_packed_kernel_r2",
                                "flux_collide_kernel", "flux_packed_inner_kernel", "flux_packed_inner_kernel_paired"};
        const int counts[5] = {h->n_reg, h->n_r2, h->n_nonreg, h->n_inner, h->n_innerp};
        const int64_t units[5] = {h->ph_reg, h->ph_r2, h->ph_nonreg, h->ph_inner, h->ph_innerp};
        for (int part = 0; part < 5; ++part) {
            if (counts[part] == 0) continue;
            begin();
            e = launch_flux_part(h, P, part, h->sched, h->sched_ctas, s, false);
            if (e != cudaSuccess) return cuda_fail(h, e, names[part]);
            end(names[part], units[part]);
        }
        *launches += (h->n_reg > 0) + (h->n_nonreg > 0) + (h->n_r2 > 0) + (h->n_inner > 0) + (h->n_innerp > 0);
        if (h->prm.marching == KG_MARCH_CIP) {
            begin();
            e = dispatch(h, [&](auto L) { return decltype(L)::cip(P, F.n_fluid, s); });
            if (e != cudaSuccess) return cuda_fail(h, e, "cip_kernel");
            end("cip_kernel");
            ++*launches;
        }
    }
    e = launch_residual(P, h->d_live, (int)h->live.size(), h->res_out, s);
    if (e != cudaSuccess) return cuda_fail(h, e, "residual_kernel");
    ++*launches;
    h->parity ^= 1;
    return KG_OK;
}

// Runs nsteps steps of all live problems; fills per-slot residual flags/sums into h_res.
int run_steps(kg_handle* h, int32_t nsteps, double* device_ms, int64_t* launches_out) {
    int rc = rebuild(h);
    if (rc) return rc;
    if (nsteps > 0 && has_lazy_slopes(h)) h->sdf_partial = true;   // the steps leave the lazy cells' sdf
    if (h->autotune && h->tuned_version != h->version) {
        rc = autotune_flux(h);
        if (rc) return rc;
    }
    // clear the checked flags so the report covers this call only
    for (int s : h->live)
        KG_CUDA(h, cudaMemsetAsync(h->res_out + (int64_t)s * RES_STRIDE + 2 * MAXW + 1, 0, sizeof(double), h->stream));
    cudaEvent_t t0, t1;
    KG_CUDA(h, cudaEventCreate(&t0));
    KG_CUDA(h, cudaEventCreate(&t1));
    KG_CUDA(h, cudaEventRecord(t0, h->stream));
    int64_t launches = 0;
    if (h->use_graph && !h->prof && nsteps > 0) {
        bool reuse = h->gexec && h->g_nsteps == nsteps && h->g_parity == h->parity && h->g_version == h->version;
        if (!reuse) {
            if (h->gexec) { cudaGraphExecDestroy(h->gexec); h->gexec = nullptr; }
            int parity0 = h->parity;
            cudaGraph_t graph;
            KG_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
            int r = KG_OK;
            int64_t l = 0;
            for (int s = 0; s < nsteps && r == KG_OK; ++s) r = enqueue_step(h, false, &l);
            cudaError_t ce = cudaStreamEndCapture(h->stream, &graph);
            h->parity = parity0;
            if (r) return r;
            if (ce != cudaSuccess) return cuda_fail(h, ce, "cudaStreamEndCapture");
            ce = cudaGraphInstantiate(&h->gexec, graph, 0);
            cudaGraphDestroy(graph);
            if (ce != cudaSuccess) return cuda_fail(h, ce, "cudaGraphInstantiate");
            h->g_nsteps = nsteps; h->g_parity = parity0; h->g_version = h->version;
            h->last_launches = l;
        }
        KG_CUDA(h, cudaGraphLaunch(h->gexec, h->stream));
        launches = h->last_launches;
        if (nsteps % 2) h->parity ^= 1;
    } else {
        for (int s = 0; s < nsteps; ++s) {
            rc = enqueue_step(h, h->prof, &launches);
            if (rc) return rc;
        }
    }
    KG_CUDA(h, cudaEventRecord(t1, h->stream));
    KG_CUDA(h, cudaMemcpyAsync(h->h_res, h->res_out, sizeof(double) * MAX_SLOTS * RES_STRIDE, cudaMemcpyDeviceToHost, h->stream));
    KG_CUDA(h, cudaMemcpyAsync(h->h_status, h->d_status, sizeof(int) * MAX_SLOTS, cudaMemcpyDeviceToHost, h->stream));
    KG_CUDA(h, cudaStreamSynchronize(h->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, t0, t1);
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    *device_ms = ms;
    *launches_out = launches;
    return KG_OK;
}

void fill_report(const kg_handle* h, int slot, double ms, int64_t launches, kg_step_report* r) {
    std::memset(r, 0, sizeof(*r));
    const double* o = h->h_res + (int64_t)slot * RES_STRIDE;
    r->checked = o[2 * MAXW + 1] != 0.0;
    r->checked_step = r->checked ? (int64_t)o[2 * MAXW] : -1;
    for (int e = 0; e < 5; ++e) { r->sum_res[e] = o[e]; r->sum_avg[e] = o[MAXW + e]; }
    r->device_ms = ms;
    r->phase_cells = h->probs[slot].F.phase_cells;
    r->kernel_launches = (int32_t)launches;
    int st = h->h_status[slot];
    r->status = st ? ((st & ST_NONFINITE) ? KG_ERR_NONFINITE : KG_ERR_NEGATIVE) : KG_OK;
}

// Pipelined serving of independent requests on the single problem (kg_serve).  Three streams:
// s_in uploads request r+1 into FP64 staging while the handle's stream steps request r and
// s_out downloads request r-1 from one of two FP64 output stagings; events order the reuse of
// each staging.  Request r: f, w, prim from the host -> the steps -> f, w, prim, qf to the
// host, the same device work as kg_upload_state + kg_step + kg_download_state.
int prepare_wall_copies(kg_handle* h, int slot);
cudaError_t launch_wall_copies(const kg_handle* h, int nwall, char* fa, cudaStream_t s);
int enqueue_step(kg_handle* h, bool timed, int64_t* launches);
int serve(kg_handle* h, int32_t n, const double* const* f_in, const double* const* w_in, const double* const* prim_in,
          double dt, int64_t step0, int32_t nsteps, double* const* f_out, double* const* w_out,
          double* const* prim_out, double* const* qf_out, kg_step_report* reports) {
    Problem& pb = h->probs[0];
    if (!pb.live) { pb.live = true; h->dirty = true; }
    int rc = rebuild(h);
    if (rc) return rc;
    if (nsteps > 0 && has_lazy_slopes(h)) h->sdf_partial = true;   // the steps leave the lazy cells' sdf
    if (h->autotune && h->tuned_version != h->version && (rc = autotune_flux(h))) return rc;
    if (pb.pp.dt != dt && (rc = set_prob_dt(h, 0, dt))) return rc;
    const Flat& L = pb.F;
    const int D = h->prm.dim, NW = D + 2, NC = L.n_cells;
    const int64_t nfc = L.foff[NC], nd = pb.dsize, fb = pb.fbase, db = pb.dbase;
    const size_t ss = storage_size(h);
    // staging: f in, two f out, rows in (w, prim), two rows out (w, prim, qf)
    const int64_t rin = 2LL * NC * NW, rout = 2LL * NC * NW + (int64_t)NC * D;
    const int64_t need = 3 * nfc + rin + 2 * rout;
    if (h->sv_cap < need) {
        if (h->sv_buf) cudaFree(h->sv_buf);
        h->sv_buf = nullptr;
        h->sv_cap = 0;
        if (cudaMalloc(&h->sv_buf, sizeof(double) * need) != cudaSuccess) {
            h->sv_buf = nullptr;
            return fail(h, KG_ERR_NOMEM, "cudaMalloc serving staging");
        }
        h->sv_cap = need;
    }
    if (!h->s_in) KG_CUDA(h, cudaStreamCreateWithFlags(&h->s_in, cudaStreamNonBlocking));
    if (!h->s_out) KG_CUDA(h, cudaStreamCreateWithFlags(&h->s_out, cudaStreamNonBlocking));
    double* d_fin = h->sv_buf;
    double* d_fout[2] = {d_fin + nfc, d_fin + 2 * nfc};
    double* d_rin = d_fin + 3 * nfc;
    double* d_rout[2] = {d_rin + rin, d_rin + rin + rout};
    if ((rc = prepare_wall_copies(h, 0))) return rc;
    const int nwall = (int)L.wall_ops.size();
    // per request: residual row and status word, copied on the device, read at the end
    double* d_rep = nullptr;
    if (cudaMalloc(&d_rep, sizeof(double) * (size_t)n * (RES_STRIDE + 1)) != cudaSuccess)
        return fail(h, KG_ERR_NOMEM, "cudaMalloc serving reports");
    std::vector<cudaEvent_t> ev((size_t)n * 6, nullptr);   // h2d, in_free, done, out_free, t0, t1
    struct Cleanup {
        std::vector<cudaEvent_t>& ev;
        double* rep;
        ~Cleanup() {
            for (cudaEvent_t e : ev) if (e) cudaEventDestroy(e);
            if (rep) cudaFree(rep);
        }
    } cleanup{ev, d_rep};
    for (int32_t r = 0; r < n; ++r)
        for (int k = 0; k < 6; ++k)
            KG_CUDA(h, cudaEventCreateWithFlags(&ev[(size_t)r * 6 + k], k < 4 ? cudaEventDisableTiming : cudaEventDefault));
    auto E = [&](int32_t r, int k) { return ev[(size_t)r * 6 + k]; };
    std::vector<int64_t> launches((size_t)n, 0);
    const int tb = 256;
    auto blocks = [&](int64_t m) { return (int)std::min<int64_t>((m + tb - 1) / tb, 1 << 20); };
    for (int32_t r = 0; r < n; ++r) {
        // upload (s_in), once the previous request has consumed the input staging
        if (r > 0) KG_CUDA(h, cudaStreamWaitEvent(h->s_in, E(r - 1, 1), 0));
        KG_CUDA(h, cudaMemcpyAsync(d_fin, f_in[r], sizeof(double) * nfc, cudaMemcpyHostToDevice, h->s_in));
        KG_CUDA(h, cudaMemcpyAsync(d_rin, w_in[r], sizeof(double) * NC * NW, cudaMemcpyHostToDevice, h->s_in));
        KG_CUDA(h, cudaMemcpyAsync(d_rin + NC * NW, prim_in[r], sizeof(double) * NC * NW, cudaMemcpyHostToDevice, h->s_in));
        KG_CUDA(h, cudaEventRecord(E(r, 0), h->s_in));
        // state (handle stream)
        cudaStream_t s = h->stream;
        KG_CUDA(h, cudaStreamWaitEvent(s, E(r, 0), 0));
        char* fa = (char*)(h->parity == 0 ? h->fA : h->fB) + fb * ss;
        if (h->prm.precision == KG_PREC_FP64)
            KG_CUDA(h, cudaMemcpyAsync(fa, d_fin, sizeof(double) * nfc, cudaMemcpyDeviceToDevice, s));
        else
            to_storage<float><<<1024, 256, 0, s>>>(d_fin, (float*)fa, nfc);
        rows_unpack<<<blocks(nd * MAXW), tb, 0, s>>>(d_rin, NW, NC, h->w + db * MAXW, MAXW, (int)nd);
        rows_unpack<<<blocks(nd * MAXW), tb, 0, s>>>(d_rin + NC * NW, NW, NC, h->prim + db * MAXW, MAXW, (int)nd);
        KG_CUDA(h, cudaGetLastError());
        KG_CUDA(h, cudaEventRecord(E(r, 1), s));
        KG_CUDA(h, launch_wall_copies(h, nwall, fa, s));
        KG_CUDA(h, cudaMemsetAsync((char*)h->sdf + fb * D * ss, 0, pb.fsize * D * ss, s));
        KG_CUDA(h, cudaMemsetAsync(h->qf + db * MAXD, 0, sizeof(double) * nd * MAXD, s));
        set_step_counter<<<1, 1, 0, s>>>(h->d_step, step0);
        KG_CUDA(h, cudaMemsetAsync(h->d_status, 0, sizeof(int), s));
        KG_CUDA(h, cudaMemsetAsync(h->res_out + 2 * MAXW + 1, 0, sizeof(double), s));
        KG_CUDA(h, cudaEventRecord(E(r, 4), s));
        for (int32_t k = 0; k < nsteps; ++k)
            if ((rc = enqueue_step(h, false, &launches[r]))) return rc;
        KG_CUDA(h, cudaEventRecord(E(r, 5), s));
        KG_CUDA(h, cudaMemcpyAsync(d_rep + (int64_t)r * (RES_STRIDE + 1), h->res_out, sizeof(double) * RES_STRIDE, cudaMemcpyDeviceToDevice, s));
        KG_CUDA(h, cudaMemcpyAsync(d_rep + (int64_t)r * (RES_STRIDE + 1) + RES_STRIDE, h->d_status, sizeof(int), cudaMemcpyDeviceToDevice, s));
        // result into output staging r % 2, once request r-2 has left it
        if (r >= 2) KG_CUDA(h, cudaStreamWaitEvent(s, E(r - 2, 3), 0));
        const char* fr = (const char*)(h->parity == 0 ? h->fA : h->fB) + fb * ss;
        double* fo = d_fout[r % 2];
        double* ro = d_rout[r % 2];
        if (h->prm.precision == KG_PREC_FP64)
            KG_CUDA(h, cudaMemcpyAsync(fo, fr, sizeof(double) * nfc, cudaMemcpyDeviceToDevice, s));
        else
            from_storage<float><<<1024, 256, 0, s>>>((const float*)fr, fo, nfc);
        rows_pack<<<blocks((int64_t)NC * NW), tb, 0, s>>>(h->w + db * MAXW, MAXW, ro, NW, NC);
        rows_pack<<<blocks((int64_t)NC * NW), tb, 0, s>>>(h->prim + db * MAXW, MAXW, ro + NC * NW, NW, NC);
        rows_pack<<<blocks((int64_t)NC * D), tb, 0, s>>>(h->qf + db * MAXD, MAXD, ro + 2 * NC * NW, D, NC);
        KG_CUDA(h, cudaGetLastError());
        KG_CUDA(h, cudaEventRecord(E(r, 2), s));
        // download (s_out)
        KG_CUDA(h, cudaStreamWaitEvent(h->s_out, E(r, 2), 0));
        if (f_out && f_out[r]) KG_CUDA(h, cudaMemcpyAsync(f_out[r], fo, sizeof(double) * nfc, cudaMemcpyDeviceToHost, h->s_out));
        if (w_out && w_out[r]) KG_CUDA(h, cudaMemcpyAsync(w_out[r], ro, sizeof(double) * NC * NW, cudaMemcpyDeviceToHost, h->s_out));
        if (prim_out && prim_out[r]) KG_CUDA(h, cudaMemcpyAsync(prim_out[r], ro + NC * NW, sizeof(double) * NC * NW, cudaMemcpyDeviceToHost, h->s_out));
        if (qf_out && qf_out[r]) KG_CUDA(h, cudaMemcpyAsync(qf_out[r], ro + 2 * NC * NW, sizeof(double) * NC * D, cudaMemcpyDeviceToHost, h->s_out));
        KG_CUDA(h, cudaEventRecord(E(r, 3), h->s_out));
    }
    KG_CUDA(h, cudaStreamSynchronize(h->s_out));
    KG_CUDA(h, cudaStreamSynchronize(h->stream));
    std::vector<double> rep((size_t)n * (RES_STRIDE + 1));
    KG_CUDA(h, cudaMemcpy(rep.data(), d_rep, sizeof(double) * rep.size(), cudaMemcpyDeviceToHost));
    h->have_state = true;
    int worst = KG_OK;
    for (int32_t r = 0; r < n; ++r) {
        const double* o = rep.data() + (size_t)r * (RES_STRIDE + 1);
        kg_step_report R;
        std::memset(&R, 0, sizeof(R));
        R.checked = o[2 * MAXW + 1] != 0.0;
        R.checked_step = R.checked ? (int64_t)o[2 * MAXW] : -1;
        for (int e = 0; e < 5; ++e) { R.sum_res[e] = o[e]; R.sum_avg[e] = o[MAXW + e]; }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, E(r, 4), E(r, 5));
        R.device_ms = ms;
        R.phase_cells = L.phase_cells;
        R.kernel_launches = (int32_t)launches[r];
        int st = 0;
        std::memcpy(&st, o + RES_STRIDE, sizeof(int));
        R.status = st ? ((st & ST_NONFINITE) ? KG_ERR_NONFINITE : KG_ERR_NEGATIVE) : KG_OK;
        if (R.status && !worst) worst = R.status;
        if (reports) reports[r] = R;
    }
    if (worst) return fail(h, worst, worst == KG_ERR_NONFINITE ? "non-finite primitive variables" : "rho <= 0 or lambda <= 0");
    return KG_OK;
}

// SolidNeighbor df starts as a copy of the donor df (Immersed_boundary.jl:290-298): one
// launch for all walls of the problem in `slot`, within the f buffer at fa (the problem's
// block of it).
// The (donor, wall, length) copies of the problem in `slot` into h->d_tri (host-synchronous).
int prepare_wall_copies(kg_handle* h, int slot) {
    const Flat& L = h->probs[slot].F;
    const int nwall = (int)L.wall_ops.size();
    if (nwall == 0) return KG_OK;
    std::vector<int64_t> tri((size_t)nwall * 3);
    for (int k = 0; k < nwall; ++k) {
        const WallOp& wo = L.wall_ops[k];
        tri[3 * k] = L.foff[wo.donor];
        tri[3 * k + 1] = L.foff[wo.data];
        tri[3 * k + 2] = L.foff[wo.data + 1] - L.foff[wo.data];
    }
    if (h->tri_cap < (int64_t)tri.size()) {
        if (h->d_tri) cudaFree(h->d_tri);
        h->d_tri = nullptr;
        h->tri_cap = 0;
        void* p = nullptr;
        cudaError_t e = cudaMalloc(&p, sizeof(int64_t) * tri.size());
        if (e != cudaSuccess) return fail(h, KG_ERR_NOMEM, "cudaMalloc wall copies");
        h->d_tri = (int64_t*)p;
        h->tri_cap = (int64_t)tri.size();
    }
    KG_CUDA(h, cudaMemcpyAsync(h->d_tri, tri.data(), sizeof(int64_t) * tri.size(), cudaMemcpyHostToDevice, h->stream));
    KG_CUDA(h, cudaStreamSynchronize(h->stream));   // tri is host memory the copy reads
    return KG_OK;
}
// The copies prepared above, within the f buffer at fa (the problem's block of it).
cudaError_t launch_wall_copies(const kg_handle* h, int nwall, char* fa, cudaStream_t s) {
    if (nwall == 0) return cudaSuccess;
    if (h->prm.precision == KG_PREC_FP64) copy_blocks<double><<<nwall, 256, 0, s>>>((double*)fa, h->d_tri);
    else copy_blocks<float><<<nwall, 256, 0, s>>>((float*)fa, h->d_tri);
    return cudaGetLastError();
}
int init_wall_blocks(kg_handle* h, int slot, char* fa) {
    int rc = prepare_wall_copies(h, slot);
    if (rc) return rc;
    KG_CUDA(h, launch_wall_copies(h, (int)h->probs[slot].F.wall_ops.size(), fa, h->stream));
    return KG_OK;
}

// Uploads a placed problem's state into its slabs (both f buffers).
int upload_problem_state(kg_handle* h, int slot, const double* f, const double* w, const double* prim, int64_t step) {
    Problem& pb = h->probs[slot];
    const int64_t nf = pb.fsize, nd = pb.dsize, fb = pb.fbase, db = pb.dbase;
    Flat& L = pb.F;
    const int D = h->prm.dim, NW = D + 2;
    const int64_t nfc = L.foff[L.n_cells];
    size_t ss = storage_size(h);
    // into the buffer the next step reads; a step writes every data item's other buffer
    // (flux: fluid cells; solid and wall kernels: both buffers of theirs)
    char* fa = (char*)(h->parity == 0 ? h->fA : h->fB) + fb * ss;
    if (h->prm.precision == KG_PREC_FP64) {
        KG_CUDA(h, cudaMemcpyAsync(fa, f, sizeof(double) * nfc, cudaMemcpyHostToDevice, h->stream));
    } else {
        double* st = h->staging + fb;
        KG_CUDA(h, cudaMemcpyAsync(st, f, sizeof(double) * nfc, cudaMemcpyHostToDevice, h->stream));
        to_storage<float><<<1024, 256, 0, h->stream>>>(st, (float*)fa, nfc);
        KG_CUDA(h, cudaGetLastError());
    }
    {
        int rc = init_wall_blocks(h, slot, fa);
        if (rc) return rc;
    }
    KG_CUDA(h, cudaMemsetAsync((char*)h->sdf + fb * D * ss, 0, nf * D * ss, h->stream));
    std::vector<double> pw((size_t)nd * MAXW, 0.0), pp((size_t)nd * MAXW, 0.0);
    for (int c = 0; c < L.n_cells; ++c)
        for (int e = 0; e < NW; ++e) { pw[(size_t)c * MAXW + e] = w[(size_t)c * NW + e]; pp[(size_t)c * MAXW + e] = prim[(size_t)c * NW + e]; }
    KG_CUDA(h, cudaMemcpyAsync(h->w + db * MAXW, pw.data(), sizeof(double) * pw.size(), cudaMemcpyHostToDevice, h->stream));
    KG_CUDA(h, cudaMemcpyAsync(h->prim + db * MAXW, pp.data(), sizeof(double) * pp.size(), cudaMemcpyHostToDevice, h->stream));
    KG_CUDA(h, cudaMemsetAsync(h->qf + db * MAXD, 0, sizeof(double) * nd * MAXD, h->stream));
    KG_CUDA(h, cudaMemcpyAsync(h->d_step + slot, &step, sizeof(int64_t), cudaMemcpyHostToDevice, h->stream));
    KG_CUDA(h, cudaMemsetAsync(h->d_status + slot, 0, sizeof(int), h->stream));
    KG_CUDA(h, cudaStreamSynchronize(h->stream));   // host temporaries
    return KG_OK;
}

// Places a flattened problem into the pools (the merged topology is rebuilt before the
// next step) and uploads its state.
int complete_last_slopes(kg_handle* h);
int place_problem(kg_handle* h, int slot, Flat&& F, const kg_params& prm, const double* f, const double* w,
                  const double* prim, double dt, int64_t step) {
    Problem& pb = h->probs[slot];
    const int64_t nf = F.foff.back();
    const int64_t nd = F.n_data;
    int64_t fb, db;
    {
        // the last step's slopes of the lazy cells of the live problems, before the layout changes
        const int rc0 = complete_last_slopes(h);
        if (rc0) return rc0;
    }
    if (!h->fslab.alloc(nf, &fb)) return fail(h, KG_ERR_BUDGET, "f pool exhausted (admission refused by footprint)");
    if (!h->dslab.alloc(nd, &db)) { h->fslab.release(fb, nf); return fail(h, KG_ERR_BUDGET, "cell pool exhausted"); }
    pb.F = std::move(F);
    pb.fbase = fb; pb.fsize = nf; pb.dbase = db; pb.dsize = nd;
    pb.pp = params_of(prm, dt);
    pb.live = true;
    h->dirty = true;
    return upload_problem_state(h, slot, f, w, prim, step);
}

int download_problem(kg_handle* h, int slot, double* f, double* w, double* prim, double* qf, double* sdf) {
    Problem& pb = h->probs[slot];
    Flat& L = pb.F;
    const int D = h->prm.dim, NW = D + 2;
    const int64_t nfc = L.foff[L.n_cells];
    size_t ss = storage_size(h);
    void* fin = h->parity == 0 ? h->fA : h->fB;
    const char* fsrc = (const char*)fin + pb.fbase * ss;
    if (f) {
        if (h->prm.precision == KG_PREC_FP64) {
            KG_CUDA(h, cudaMemcpyAsync(f, fsrc, sizeof(double) * nfc, cudaMemcpyDeviceToHost, h->stream));
        } else {
            double* st = h->staging + pb.fbase;
            from_storage<float><<<1024, 256, 0, h->stream>>>((const float*)fsrc, st, nfc);
            KG_CUDA(h, cudaGetLastError());
            KG_CUDA(h, cudaMemcpyAsync(f, st, sizeof(double) * nfc, cudaMemcpyDeviceToHost, h->stream));
        }
    }
    if (sdf) {
        { const int rc2 = complete_last_slopes(h); if (rc2) return rc2; }
        const char* ssrc = (const char*)h->sdf + pb.fbase * D * ss;
        if (h->prm.precision == KG_PREC_FP64) {
            KG_CUDA(h, cudaMemcpyAsync(sdf, ssrc, sizeof(double) * nfc * D, cudaMemcpyDeviceToHost, h->stream));
        } else {
            double* st = h->staging + pb.fbase;   // the problem's staging slab holds nf >= nfc doubles
            for (int d = 0; d < D; ++d) {
                from_storage<float><<<1024, 256, 0, h->stream>>>((const float*)ssrc + (int64_t)d * nfc, st, nfc);
                KG_CUDA(h, cudaGetLastError());
                KG_CUDA(h, cudaMemcpyAsync(sdf + (int64_t)d * nfc, st, sizeof(double) * nfc, cudaMemcpyDeviceToHost, h->stream));
                KG_CUDA(h, cudaStreamSynchronize(h->stream));
            }
        }
    }
    const int64_t nd = pb.dsize;
    std::vector<double> pw((size_t)nd * MAXW), pp((size_t)nd * MAXW), pq((size_t)nd * MAXD);
    if (w) KG_CUDA(h, cudaMemcpyAsync(pw.data(), h->w + pb.dbase * MAXW, sizeof(double) * pw.size(), cudaMemcpyDeviceToHost, h->stream));
    if (prim) KG_CUDA(h, cudaMemcpyAsync(pp.data(), h->prim + pb.dbase * MAXW, sizeof(double) * pp.size(), cudaMemcpyDeviceToHost, h->stream));
    if (qf) KG_CUDA(h, cudaMemcpyAsync(pq.data(), h->qf + pb.dbase * MAXD, sizeof(double) * pq.size(), cudaMemcpyDeviceToHost, h->stream));
    KG_CUDA(h, cudaStreamSynchronize(h->stream));
    for (int c = 0; c < L.n_cells; ++c) {
        for (int e = 0; e < NW; ++e) {
            if (w) w[(size_t)c * NW + e] = pw[(size_t)c * MAXW + e];
            if (prim) prim[(size_t)c * NW + e] = pp[(size_t)c * MAXW + e];
        }
        if (qf) for (int d = 0; d < D; ++d) qf[(size_t)c * D + d] = pq[(size_t)c * MAXD + d];
    }
    return KG_OK;
}

// sw of the problem in `slot` (update_macro_slope!) from the slopes on the device, into a
// device array of (dim+2) x dim doubles per data item of the problem (zero rows for items
// without a fluid-list entry); or, for the physical-space criterion, fresh slopes of the
// current f, their sw and the criterion with the buffer layer (update_criterion! +
// apply_amr_buffer!) into a second such array.  The host receives the rows of the problem's
// cells.
int sync_point_rows(kg_handle* h, int slot, double* sw_host, double thr, double* loh_host) {
    int rc = rebuild(h);
    if (rc) return rc;
    Problem& pb = h->probs[slot];
    const int D = h->prm.dim, N = D * (D + 2);
    const int fb = pb.pp.fluid_begin, n = pb.pp.fluid_end - pb.pp.fluid_begin;
    const int64_t nd = pb.dsize, nc = pb.F.n_cells;
    const size_t bytes = sizeof(double) * (size_t)std::max<int64_t>(nd, 1) * N;
    double* d = nullptr;
    cudaError_t e = cudaMalloc(&d, 3 * bytes);
    if (e != cudaSuccess) return fail(h, KG_ERR_NOMEM, "cudaMalloc sync-point rows");
    double* dsw = d;
    double* dloh = d + bytes / sizeof(double);
    double* dout = dloh + bytes / sizeof(double);
    Dev P = h->dev;
    P.f_in = h->parity == 0 ? h->fA : h->fB;
    P.f_out = h->parity == 0 ? h->fB : h->fA;
    e = cudaMemsetAsync(d, 0, 3 * bytes, h->stream);
    // ps_adaptive_mesh_refinement! (Physical_space/AMR.jl:1108-1116) runs slope! on the current
    // f before update_criterion!; the next step recomputes the same slopes, so the state a step
    // sees is unchanged (in a batch the pass covers every live problem)
    if (e == cudaSuccess && loh_host) e = enqueue_slopes_full(h, P, h->stream);
    if (e == cudaSuccess && !loh_host) {
        // sw of the slopes the last step used
        const int rc2 = complete_last_slopes(h);
        if (rc2) { cudaFree(d); return rc2; }
    }
    if (e == cudaSuccess)
        e = dispatch(h, [&](auto L) { return decltype(L)::macro_slope(P, fb, n, (int)pb.dbase, dsw, h->stream); });
    if (e == cudaSuccess && loh_host)
        e = dispatch(h, [&](auto L) { return decltype(L)::criterion(P, fb, n, (int)pb.dbase, dsw, thr, dloh, dout, h->stream); });
    if (e == cudaSuccess && sw_host)
        e = cudaMemcpyAsync(sw_host, dsw, sizeof(double) * (size_t)nc * N, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess && loh_host)
        e = cudaMemcpyAsync(loh_host, dout, sizeof(double) * (size_t)nc * N, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(h, e, "sync-point rows");
    return KG_OK;
}

// ---- physical-space adaptation (ps_replace!, Physical_space/AMR.jl:633-703) -----------
// Same velocity grid content (levels, weights, midpoints) of grid ga of A and grid gb of B.
bool same_grid(const Flat& A, int ga, const Flat& B, int gb) {
    const int64_t na = A.g_off[ga + 1] - A.g_off[ga], nb = B.g_off[gb + 1] - B.g_off[gb];
    if (na != nb) return false;
    const int64_t a0 = A.g_off[ga], b0 = B.g_off[gb];
    const int64_t PA = (int64_t)A.vw.size(), PB = (int64_t)B.vw.size();
    if (std::memcmp(&A.vlev[a0], &B.vlev[b0], (size_t)na) != 0) return false;
    if (std::memcmp(&A.vw[a0], &B.vw[b0], sizeof(double) * (size_t)na) != 0) return false;
    for (int d = 0; d < A.dim; ++d)
        if (std::memcmp(&A.vu[(size_t)d * PA + a0], &B.vu[(size_t)d * PB + b0], sizeof(double) * (size_t)na) != 0) return false;
    return true;
}

struct AdaptPlan {
    std::vector<AdaptRec> recs;
    std::vector<int32_t> runs;   // (j0, count) pairs
    std::vector<int8_t> lev;     // levels of the children's grids that need runs
};

// Checks the per-cell sources of the adapted mesh Fn (placed at data slot dbn) against the
// previous mesh Fo (placed at fbo / dbo) and resolves them to pool positions.
int build_adapt_plan(kg_handle* h, const Flat& Fo, int64_t fbo, int64_t dbo, const Flat& Fn, int64_t dbn,
                     const kg_adapt_src* src, AdaptPlan& plan) {
    const int D = Fn.dim, NC = Fn.n_cells, NCo = Fo.n_cells, nch = 1 << D;
    std::map<std::pair<int, int>, bool> same;                 // (previous grid, new grid)
    std::map<std::pair<int, int>, int64_t> run_of;            // (new grid, previous grid) -> first pair
    std::map<int, int64_t> lev_of;                            // previous grid -> level table offset
    auto is_same = [&](int go, int gn) {
        auto key = std::make_pair(go, gn);
        auto it = same.find(key);
        if (it != same.end()) return it->second;
        const bool r = same_grid(Fo, go, Fn, gn);
        same[key] = r;
        return r;
    };
    auto where = [](int c) { return " (new cell " + std::to_string(c) + ")"; };
    std::vector<int32_t> tmp;
    plan.recs.assign(NC, AdaptRec{});
    for (int c = 0; c < NC; ++c) {
        const kg_adapt_src& a = src[c];
        AdaptRec& r = plan.recs[c];
        r.cell = (int32_t)(dbn + c);
        r.kind = a.kind;
        const int gn = Fn.dgrid[c];
        for (int q = 0; q < 8; ++q) r.run[q] = -1;
        if (a.kind == KG_ADAPT_KEEP || a.kind == KG_ADAPT_REFINE) {
            const int o = a.src[0];
            if (o < 0 || o >= NCo) return fail(h, KG_ERR_ARG, "adapt source cell out of range" + where(c));
            if (!is_same(Fo.dgrid[o], gn))
                return fail(h, KG_ERR_TOPOLOGY, "a kept or refined cell must keep its source's velocity grid" + where(c));
            r.nsrc = 1;
            r.src_f[0] = fbo + Fo.foff[o];
            r.src_nv[0] = Fo.dnv[o];
            r.src_d[0] = (int32_t)(dbo + o);
            if (a.kind == KG_ADAPT_REFINE) {
                if (a.depth < 1 || a.depth > KG_ADAPT_MAX_DEPTH) return fail(h, KG_ERR_ARG, "refinement depth out of range" + where(c));
                r.depth = a.depth;
                for (int l = 0; l < a.depth; ++l) {
                    if (a.path[l] < 0 || a.path[l] >= nch) return fail(h, KG_ERR_ARG, "child number out of range" + where(c));
                    r.path[l] = a.path[l];
                }
                for (int d = 0; d < D; ++d) r.ds[d] = Fo.dds[(size_t)o * MAXD + d];
            }
        } else if (a.kind == KG_ADAPT_COARSEN) {
            int best = 0;
            for (int q = 0; q < nch; ++q) {
                const int o = a.src[q];
                if (o < 0 || o >= NCo) return fail(h, KG_ERR_ARG, "adapt source cell out of range" + where(c));
                if (Fo.dnv[o] < Fo.dnv[a.src[best]]) best = q;
            }
            // ps_merge keeps the grid of the first child with the fewest velocity cells
            if (!is_same(Fo.dgrid[a.src[best]], gn))
                return fail(h, KG_ERR_TOPOLOGY, "a coarsened cell takes the grid of its first child with the fewest velocity cells" + where(c));
            r.nsrc = nch;
            for (int q = 0; q < nch; ++q) {
                const int o = a.src[q], go = Fo.dgrid[o];
                r.src_f[q] = fbo + Fo.foff[o];
                r.src_nv[q] = Fo.dnv[o];
                r.src_d[q] = (int32_t)(dbo + o);
                if (is_same(go, gn)) continue;
                auto key = std::make_pair(gn, go);
                auto it = run_of.find(key);
                if (it == run_of.end()) {
                    const int64_t nn = Fn.g_off[gn + 1] - Fn.g_off[gn], no = Fo.g_off[go + 1] - Fo.g_off[go];
                    if (!level_runs(&Fn.vlev[Fn.g_off[gn]], (int)nn, &Fo.vlev[Fo.g_off[go]], (int)no, D, tmp))
                        return fail(h, KG_ERR_TOPOLOGY, "velocity grids of a coarsening do not tile the same root lattice" + where(c));
                    it = run_of.emplace(key, (int64_t)plan.runs.size() / 2).first;
                    plan.runs.insert(plan.runs.end(), tmp.begin(), tmp.end());
                }
                r.run[q] = it->second;
                auto lt = lev_of.find(go);
                if (lt == lev_of.end()) {
                    lt = lev_of.emplace(go, (int64_t)plan.lev.size()).first;
                    plan.lev.insert(plan.lev.end(), Fo.vlev.begin() + Fo.g_off[go], Fo.vlev.begin() + Fo.g_off[go + 1]);
                }
                r.lev[q] = lt->second;
            }
        } else if (a.kind == KG_ADAPT_VS) {
            const int o = a.src[0];
            if (o < 0 || o >= NCo) return fail(h, KG_ERR_ARG, "adapt source cell out of range" + where(c));
            const int go = Fo.dgrid[o];
            r.nsrc = 1;
            r.src_f[0] = fbo + Fo.foff[o];
            r.src_nv[0] = Fo.dnv[o];
            r.src_d[0] = (int32_t)(dbo + o);
            if (!is_same(go, gn)) {
                auto key = std::make_pair(gn, go);
                auto it = run_of.find(key);
                if (it == run_of.end()) {
                    const int64_t nn = Fn.g_off[gn + 1] - Fn.g_off[gn], no = Fo.g_off[go + 1] - Fo.g_off[go];
                    if (!level_runs(&Fn.vlev[Fn.g_off[gn]], (int)nn, &Fo.vlev[Fo.g_off[go]], (int)no, D, tmp))
                        return fail(h, KG_ERR_TOPOLOGY, "a rebuilt velocity grid does not tile its source grid's root lattice" + where(c));
                    it = run_of.emplace(key, (int64_t)plan.runs.size() / 2).first;
                    plan.runs.insert(plan.runs.end(), tmp.begin(), tmp.end());
                }
                r.run[0] = it->second;
                auto lt = lev_of.find(go);
                if (lt == lev_of.end()) {
                    lt = lev_of.emplace(go, (int64_t)plan.lev.size()).first;
                    plan.lev.insert(plan.lev.end(), Fo.vlev.begin() + Fo.g_off[go], Fo.vlev.begin() + Fo.g_off[go + 1]);
                }
                r.lev[0] = lt->second;
            }
        } else {
            return fail(h, KG_ERR_ARG, "unknown adapt kind" + where(c));
        }
    }
    return KG_OK;
}

// Replaces the problem in `slot` by the adapted mesh `topo`, its state interpolated on the
// device from the previous one.  Single handle: the previous pools stay alive until the new
// ones are filled.  Batch: the new slabs are placed beside the previous ones in the shared
// pools, then the previous ones are released.
// With profiling on, host wall time of the phases of an adaptation (ms, into the profile table).

int adapt_problem(kg_handle* h, int slot, const kg_topology* topo, const kg_adapt_src* src) {
    PhaseClock clk{h};
    Flat Fn = std::move(h->spare);
    DevLayout dln;
    std::string err;
    int rc = build_layout(h, *topo, slot, Fn, dln, err);
    clk.mark("adapt:flatten");
    if (rc) return fail(h, rc, err);
    if (Fn.max_inc > MAX_INC) return fail(h, KG_ERR_TOPOLOGY, "a cell has more face incidences than supported");
    // ps_adaptive_mesh_refinement! runs slope! before the replacements read the slopes
    if ((rc = rebuild(h))) return rc;
    {
        Dev P = h->dev;
        P.f_in = h->parity == 0 ? h->fA : h->fB;
        P.f_out = h->parity == 0 ? h->fB : h->fA;
        KG_CUDA(h, enqueue_slopes_full(h, P, h->stream));
    }
    KG_CUDA(h, cudaStreamSynchronize(h->stream));
    clk.mark("adapt:slopes");
    // every check before the handle changes: a rejected adaptation leaves it as it was
    AdaptPlan plan;
    if ((rc = build_adapt_plan(h, h->probs[slot].F, h->probs[slot].fbase, h->probs[slot].dbase, Fn, 0, src, plan))) return rc;
    clk.mark("adapt:plan");
    Problem old = std::move(h->probs[slot]);
    h->probs[slot] = Problem();
    // the previous state: pointers into pools that stay alive until the end of this call
    const void* of = h->parity == 0 ? h->fA : h->fB;
    const void* osdf = h->sdf;
    const double *ow = h->w, *oprim = h->prim, *oqf = h->qf;
    kg_handle::PoolSet prev;
    const int64_t nf = Fn.foff.back(), nd = Fn.n_data;
    if (!h->is_batch) {
        // hand the previous pools over to this call, then take the spare pools of an earlier
        // adaptation when they hold the new mesh, or new ones with room for a mesh an eighth
        // larger (both clear the slot table)
        prev = take_pools(h);
        kg_handle::PoolSet& sp = h->spare_pools;
        if (!sp.allocs.empty() && sp.fcap >= nf && sp.dcap >= nd) {
            rc = adopt_pools(h, sp);
        } else {
            release_pools(sp);
            rc = make_pools(h, nf + nf / 8, nd + nd / 8);
        }
        if (rc) { release_pools(prev); return rc; }
        Problem& pn = h->probs[slot];
        h->fslab.alloc(nf, &pn.fbase);
        h->dslab.alloc(nd, &pn.dbase);
    } else {
        int64_t fb, db;
        if (!h->fslab.alloc(nf, &fb)) { h->probs[slot] = std::move(old); return fail(h, KG_ERR_BUDGET, "f pool cannot hold the adapted problem beside the previous one"); }
        if (!h->dslab.alloc(nd, &db)) {
            h->fslab.release(fb, nf);
            h->probs[slot] = std::move(old);
            return fail(h, KG_ERR_BUDGET, "cell pool cannot hold the adapted problem beside the previous one");
        }
        h->probs[slot].fbase = fb; h->probs[slot].dbase = db;
    }
    Problem& pb = h->probs[slot];
    pb.F = std::move(Fn);
    pb.dl = dln;
    pb.fsize = nf; pb.dsize = nd;
    pb.pp = old.pp;
    pb.live = true;
    h->dirty = true;
    for (AdaptRec& r : plan.recs) r.cell += (int32_t)pb.dbase;
    clk.mark("adapt:pools");
    rc = rebuild(h);
    clk.mark("adapt:rebuild");
    void* tab = nullptr;
    if (rc == KG_OK) {
        const size_t b_recs = sizeof(AdaptRec) * plan.recs.size();
        const size_t b_runs = sizeof(int32_t) * std::max<size_t>(plan.runs.size(), 2);
        const size_t b_lev = std::max<size_t>(plan.lev.size(), 16);
        const size_t o_runs = (b_recs + 255) / 256 * 256, o_lev = o_runs + (b_runs + 255) / 256 * 256;
        cudaError_t e = cudaMalloc(&tab, o_lev + b_lev);
        if (e != cudaSuccess) { tab = nullptr; rc = fail(h, KG_ERR_NOMEM, "cudaMalloc adaptation tables"); }
        else {
            char* t = (char*)tab;
            e = cudaMemcpyAsync(t, plan.recs.data(), b_recs, cudaMemcpyHostToDevice, h->stream);
            if (e == cudaSuccess && !plan.runs.empty())
                e = cudaMemcpyAsync(t + o_runs, plan.runs.data(), sizeof(int32_t) * plan.runs.size(), cudaMemcpyHostToDevice, h->stream);
            if (e == cudaSuccess && !plan.lev.empty())
                e = cudaMemcpyAsync(t + o_lev, plan.lev.data(), plan.lev.size(), cudaMemcpyHostToDevice, h->stream);
            Dev P = h->dev;
            P.f_in = h->parity == 0 ? h->fA : h->fB;
            P.f_out = h->parity == 0 ? h->fB : h->fA;
            if (e == cudaSuccess)
                e = dispatch(h, [&](auto L) {
                    return decltype(L)::adapt(P, (int)plan.recs.size(), (const AdaptRec*)t, of, osdf, ow, oprim, oqf,
                                              (const int32_t*)(t + o_runs), (const int8_t*)(t + o_lev), h->stream);
                });
            if (e == cudaSuccess) e = cudaMemsetAsync(h->d_status + slot, 0, sizeof(int), h->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
            if (e != cudaSuccess) rc = cuda_fail(h, e, "adapt_kernel");
        }
    }
    if (rc == KG_OK) {
        char* fa = (char*)(h->parity == 0 ? h->fA : h->fB) + pb.fbase * storage_size(h);
        rc = init_wall_blocks(h, slot, fa);
    }
    cudaStreamSynchronize(h->stream);
    clk.mark("adapt:move");
    if (tab) cudaFree(tab);
    h->spare = std::move(old.F);
    if (!h->is_batch) {
        // the previous pools become the spare set of the next adaptation
        if (rc == KG_OK) h->spare_pools = std::move(prev);
        else release_pools(prev);
        clk.mark("adapt:release");
        if (rc) { free_pools(h); return rc; }
        h->have_state = true;
    } else {
        h->fslab.release(old.fbase, old.fsize);
        h->dslab.release(old.dbase, old.dsize);
        clk.mark("adapt:release");
        if (rc) {
            // the problem cannot continue in a half-built state: release it
            h->fslab.release(pb.fbase, pb.fsize);
            h->dslab.release(pb.dbase, pb.dsize);
            pb = Problem();
            h->dirty = true;
            return rc;
        }
    }
    return KG_OK;
}

// ---- checkpoint payload (save_for_restart / restart, IO/Restart.jl) ----------------------
int check_quads(kg_handle* h, const Flat& L, const int32_t* quad_index, int32_t n_quads) {
    if (!quad_index) {
        if (n_quads != L.n_cells) return fail(h, KG_ERR_ARG, "without quad_index, n_quads must equal the number of cells");
        return KG_OK;
    }
    if (n_quads < L.n_cells) return fail(h, KG_ERR_ARG, "n_quads is smaller than the number of cells");
    std::vector<char> seen((size_t)n_quads, 0);
    for (int c = 0; c < L.n_cells; ++c) {
        const int32_t q = quad_index[c];
        if (q < 0 || q >= n_quads || seen[q]) return fail(h, KG_ERR_ARG, "quad_index out of range or repeated");
        seen[q] = 1;
    }
    return KG_OK;
}

// A device buffer of n doubles for the checkpoint matrix: the problem's staging slab in the
// mixed form, a temporary allocation in FP64 (*tmp is then set and must be freed).
int restart_buffer(kg_handle* h, const Problem& pb, int64_t n, double** buf, void** tmp) {
    *tmp = nullptr;
    if (h->staging && n <= pb.fsize) { *buf = h->staging + pb.fbase; return KG_OK; }
    cudaError_t e = cudaMalloc(tmp, sizeof(double) * (size_t)std::max<int64_t>(n, 1));
    if (e != cudaSuccess) { *tmp = nullptr; return fail(h, KG_ERR_NOMEM, "cudaMalloc checkpoint buffer"); }
    *buf = (double*)*tmp;
    return KG_OK;
}

int download_restart(kg_handle* h, int slot, const int32_t* quad_index, int32_t n_quads, double* vs_df, double* ws) {
    int rc;
    Problem& pb = h->probs[slot];
    const Flat& L = pb.F;
    if ((rc = check_quads(h, L, quad_index, n_quads))) return rc;
    const int D = h->prm.dim, NDF = h->prm.ndf, NW = D + 2, NC = L.n_cells;
    const int64_t nv_total = L.foff[NC] / NDF;
    if (vs_df) {
        double* buf = nullptr;
        void* tmp = nullptr;
        if ((rc = restart_buffer(h, pb, NDF * nv_total, &buf, &tmp))) return rc;
        const int64_t* dfo = nullptr;
        void* fo = nullptr;
        cudaError_t e = cudaMalloc(&fo, sizeof(int64_t) * (NC + 1));
        if (e == cudaSuccess) {
            dfo = (const int64_t*)fo;
            e = cudaMemcpyAsync(fo, L.foff.data(), sizeof(int64_t) * (NC + 1), cudaMemcpyHostToDevice, h->stream);
        }
        const size_t ss = storage_size(h);
        const char* fin = (const char*)(h->parity == 0 ? h->fA : h->fB) + pb.fbase * ss;
        const int grid = std::min(NC, 152 * 8);
        if (e == cudaSuccess) {
            if (h->prm.precision == KG_PREC_FP64) restart_gather<double><<<grid, 256, 0, h->stream>>>((const double*)fin, dfo, NC, NDF, nv_total, buf);
            else restart_gather<float><<<grid, 256, 0, h->stream>>>((const float*)fin, dfo, NC, NDF, nv_total, buf);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(vs_df, buf, sizeof(double) * NDF * nv_total, cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (fo) cudaFree(fo);
        if (tmp) cudaFree(tmp);
        if (e != cudaSuccess) return cuda_fail(h, e, "restart gather");
    }
    if (ws) {
        std::vector<double> pw((size_t)pb.dsize * MAXW);
        KG_CUDA(h, cudaMemcpyAsync(pw.data(), h->w + pb.dbase * MAXW, sizeof(double) * pw.size(), cudaMemcpyDeviceToHost, h->stream));
        KG_CUDA(h, cudaStreamSynchronize(h->stream));
        std::fill(ws, ws + (size_t)n_quads * NW, 0.0);
        for (int c = 0; c < NC; ++c) {
            const int64_t q = quad_index ? quad_index[c] : c;
            for (int e = 0; e < NW; ++e) ws[(size_t)e * n_quads + q] = pw[(size_t)c * MAXW + e];
        }
    }
    return KG_OK;
}

int upload_restart(kg_handle* h, int slot, const int32_t* quad_index, int32_t n_quads, const double* vs_df,
                   const double* ws, int64_t step) {
    int rc;
    Problem& pb = h->probs[slot];
    const Flat& L = pb.F;
    if ((rc = check_quads(h, L, quad_index, n_quads))) return rc;
    const int D = h->prm.dim, NDF = h->prm.ndf, NW = D + 2, NC = L.n_cells;
    const int64_t nv_total = L.foff[NC] / NDF;
    const size_t ss = storage_size(h);
    char* fa = (char*)(h->parity == 0 ? h->fA : h->fB) + pb.fbase * ss;
    double* buf = nullptr;
    void* tmp = nullptr;
    if ((rc = restart_buffer(h, pb, NDF * nv_total, &buf, &tmp))) return rc;
    void* fo = nullptr;
    cudaError_t e = cudaMalloc(&fo, sizeof(int64_t) * (NC + 1));
    if (e == cudaSuccess) e = cudaMemcpyAsync(fo, L.foff.data(), sizeof(int64_t) * (NC + 1), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(buf, vs_df, sizeof(double) * NDF * nv_total, cudaMemcpyHostToDevice, h->stream);
    const int grid = std::min(NC, 152 * 8);
    if (e == cudaSuccess) {
        if (h->prm.precision == KG_PREC_FP64) restart_scatter<double><<<grid, 256, 0, h->stream>>>(buf, (const int64_t*)fo, NC, NDF, nv_total, (double*)fa);
        else restart_scatter<float><<<grid, 256, 0, h->stream>>>(buf, (const int64_t*)fo, NC, NDF, nv_total, (float*)fa);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (fo) cudaFree(fo);
    if (tmp) cudaFree(tmp);
    if (e != cudaSuccess) return cuda_fail(h, e, "restart scatter");
    if ((rc = init_wall_blocks(h, slot, fa))) return rc;
    // w from ws; prim = get_prim(w) on the device; slopes and qf zero (restart's PsData)
    std::vector<double> pw((size_t)pb.dsize * MAXW, 0.0);
    for (int c = 0; c < NC; ++c) {
        const int64_t q = quad_index ? quad_index[c] : c;
        for (int k = 0; k < NW; ++k) pw[(size_t)c * MAXW + k] = ws[(size_t)k * n_quads + q];
    }
    KG_CUDA(h, cudaMemcpyAsync(h->w + pb.dbase * MAXW, pw.data(), sizeof(double) * pw.size(), cudaMemcpyHostToDevice, h->stream));
    KG_CUDA(h, cudaMemsetAsync(h->prim + pb.dbase * MAXW, 0, sizeof(double) * pb.dsize * MAXW, h->stream));
    if (D == 2) prim_of_w<2><<<(NC + 127) / 128, 128, 0, h->stream>>>(h->w + pb.dbase * MAXW, h->prim + pb.dbase * MAXW, NC, pb.pp.gamma);
    else prim_of_w<3><<<(NC + 127) / 128, 128, 0, h->stream>>>(h->w + pb.dbase * MAXW, h->prim + pb.dbase * MAXW, NC, pb.pp.gamma);
    KG_CUDA(h, cudaGetLastError());
    KG_CUDA(h, cudaMemsetAsync((char*)h->sdf + pb.fbase * D * ss, 0, pb.fsize * D * ss, h->stream));
    KG_CUDA(h, cudaMemsetAsync(h->qf + pb.dbase * MAXD, 0, sizeof(double) * pb.dsize * MAXD, h->stream));
    KG_CUDA(h, cudaMemcpyAsync(h->d_step + slot, &step, sizeof(int64_t), cudaMemcpyHostToDevice, h->stream));
    KG_CUDA(h, cudaMemsetAsync(h->d_status + slot, 0, sizeof(int), h->stream));
    KG_CUDA(h, cudaStreamSynchronize(h->stream));   // host temporaries
    return KG_OK;
}

// ---- velocity-space adaptation flags (vs_refine! / vs_coarsen!) -----------------------------
// vs_conserved_correction! (Velocity_space/AMR.jl:122-137): the I-projection of every flagged
// fluid cell of the problem in `slot` onto its w, on the device state.
int vs_conserve(kg_handle* h, int slot, const uint8_t* cell_flags) {
    int rc = rebuild(h);
    if (rc) return rc;
    const Problem& pb = h->probs[slot];
    const Flat& M = h->M;
    std::vector<int32_t> list;
    for (int k = pb.pp.fluid_begin; k < pb.pp.fluid_end; ++k) {
        const int64_t c = (int64_t)M.fluid_cells[k] - pb.dbase;
        if (c >= 0 && c < pb.F.n_cells && cell_flags[c]) list.push_back(k);
    }
    if (list.empty()) return KG_OK;
    int32_t* d_list = nullptr;
    KG_CUDA(h, cudaMalloc(&d_list, sizeof(int32_t) * list.size()));
    Dev P = h->dev;
    P.f_in = h->parity == 0 ? h->fA : h->fB;
    P.f_out = h->parity == 0 ? h->fB : h->fA;
    cudaError_t e = cudaMemcpyAsync(d_list, list.data(), sizeof(int32_t) * list.size(), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->d_status + slot, 0, sizeof(int), h->stream);
    if (e == cudaSuccess) e = dispatch(h, [&](auto L) { return decltype(L)::conserve(P, d_list, (int)list.size(), h->stream); });
    int st = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&st, h->d_status + slot, sizeof(int), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(d_list);
    if (e != cudaSuccess) return cuda_fail(h, e, "conserve_kernel");
    if (st) return fail(h, KG_ERR_NONFINITE, "non-finite I-projection multipliers");
    return KG_OK;
}

int vs_flags(kg_handle* h, int slot, const kg_vs_config* cfg, uint8_t* flags, double* eta, double* vr_out) {
    // the flags read the slopes the last step used
    { int rc0 = rebuild(h); if (rc0) return rc0; }
    { int rc0 = complete_last_slopes(h); if (rc0) return rc0; }
    const int D = h->prm.dim, NDF = h->prm.ndf;
    if (cfg->maxlevel < 0 || cfg->maxlevel > 12) return fail(h, KG_ERR_ARG, "maxlevel out of range");
    if (cfg->mode != KG_VS_LOHNER && cfg->mode != KG_VS_CONTRIBUTION) return fail(h, KG_ERR_ARG, "bad mode");
    double vmin[MAXD] = {0, 0, 0}, du[MAXD] = {0, 0, 0}, hf[MAXD] = {0, 0, 0};
    for (int d = 0; d < D; ++d) {
        if (cfg->vs_trees_num[d] <= 0 || !(cfg->quadrature[2 * d + 1] > cfg->quadrature[2 * d]))
            return fail(h, KG_ERR_ARG, "bad quadrature or vs_trees_num");
        if (((int64_t)cfg->vs_trees_num[d] << cfg->maxlevel) >= (int64_t(1) << 20))
            return fail(h, KG_ERR_ARG, "more than 2^20 finest velocity cells along a dimension");
        vmin[d] = cfg->quadrature[2 * d];
        du[d] = cfg->quadrature[2 * d + 1] - cfg->quadrature[2 * d];
        hf[d] = du[d] / cfg->vs_trees_num[d] / std::ldexp(1.0, cfg->maxlevel);
    }
    int rc = rebuild(h);
    if (rc) return rc;
    Problem& pb = h->probs[slot];
    const Flat& L = pb.F;
    const int c0 = (int)pb.dbase, nc = L.n_cells;
    const int64_t nv_total = L.foff[nc] / NDF;
    Dev P = h->dev;
    P.f_in = h->parity == 0 ? h->fA : h->fB;
    P.f_out = h->parity == 0 ? h->fB : h->fA;
    // vs_resolution: per-cell maxima on the device, the maximum over the fluid cells here
    std::vector<double> res((size_t)nc * 2);
    double* d_res = nullptr;
    KG_CUDA(h, cudaMalloc(&d_res, sizeof(double) * std::max(nc, 1) * 2));
    cudaError_t e = dispatch(h, [&](auto Lc) { return decltype(Lc)::vs_resolution(P, c0, nc, d_res, h->stream); });
    if (e == cudaSuccess) e = cudaMemcpyAsync(res.data(), d_res, sizeof(double) * nc * 2, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(d_res);
    if (e != cudaSuccess) return cuda_fail(h, e, "vs_resolution_kernel");
    double pdu = du[0], ptn = cfg->vs_trees_num[0];
    for (int d = 1; d < D; ++d) { pdu *= du[d]; ptn *= cfg->vs_trees_num[d]; }
    const double rweight = pdu / ptn / std::ldexp(1.0, D * cfg->maxlevel);
    double dens_res = 0.0, en_res = 0.0;
    for (int c = 0; c < nc; ++c) {
        if (L.dbe[c] < 0) continue;
        dens_res = std::max(res[2 * c] * rweight, dens_res);
        en_res = std::max(0.5 * res[2 * c + 1] * rweight, en_res);
    }
    if (vr_out) { vr_out[0] = dens_res; vr_out[1] = en_res; }
    // face neighbours of every grid of the layout (host), then the flags (device)
    const bool lohner = cfg->mode == KG_VS_LOHNER;
    std::vector<int32_t> nbr;
    if (lohner) vs_face_table(h->M, vmin, hf, cfg->vs_trees_num, cfg->maxlevel, nbr);
    else nbr.assign(1, -1);
    void* buf = nullptr;
    const size_t b_nbr = sizeof(int32_t) * nbr.size(), b_fl = (size_t)std::max<int64_t>(nv_total, 1);
    const size_t b_eta = eta ? sizeof(double) * std::max<int64_t>(nv_total, 1) : 0;
    const size_t o_fl = (b_nbr + 255) / 256 * 256, o_eta = o_fl + (b_fl + 255) / 256 * 256;
    KG_CUDA(h, cudaMalloc(&buf, o_eta + b_eta));
    char* bb = (char*)buf;
    VsFlagArgs A{};
    A.nbr = (const int32_t*)bb;
    A.flags = (uint8_t*)(bb + o_fl);
    A.eta = eta ? (double*)(bb + o_eta) : nullptr;
    A.row0 = h->M.foff[c0];
    for (int d = 0; d < MAXD; ++d) A.hf[d] = hf[d];
    A.dens_res = dens_res; A.en_res = en_res;
    A.tau_l = cfg->coeffi_lohner; A.tau_c = 0.3 * cfg->coeffi_lohner;   // VS_LOHNER_COARSEN_RATIO
    A.c_local = cfg->coeffi_local; A.c_global = cfg->coeffi_global;
    A.maxlevel = cfg->maxlevel; A.lohner = lohner ? 1 : 0;
    e = cudaMemcpyAsync(bb, nbr.data(), b_nbr, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = dispatch(h, [&](auto Lc) { return decltype(Lc)::vs_flags(P, c0, nc, A, h->stream); });
    if (e == cudaSuccess) e = cudaMemcpyAsync(flags, A.flags, (size_t)nv_total, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess && eta) e = cudaMemcpyAsync(eta, A.eta, sizeof(double) * nv_total, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(buf);
    if (e != cudaSuccess) return cuda_fail(h, e, "vs_flags_kernel");
    return KG_OK;
}

int check_params(const kg_params* params, std::string& err) {
    if (!(params->dim == 2 && params->ndf == 2) && !(params->dim == 3 && params->ndf == 1)) { err = "supported forms: dim 2 / ndf 2 and dim 3 / ndf 1"; return KG_ERR_ARG; }
    if (params->precision != KG_PREC_FP64 && params->precision != KG_PREC_MIXED) { err = "bad precision"; return KG_ERR_ARG; }
    if (params->flux != KG_FLUX_CAIDVM && params->flux != KG_FLUX_DVM) { err = "bad flux"; return KG_ERR_ARG; }
    if (params->marching != KG_MARCH_CAIDVM && params->marching != KG_MARCH_EULER && params->marching != KG_MARCH_CIP) { err = "bad marching"; return KG_ERR_ARG; }
    if (params->st_check_interval <= 0) { err = "st_check_interval must be positive"; return KG_ERR_ARG; }
    return KG_OK;
}

int create_handle(const kg_params* params, int device, kg_handle** out) {
    if (!params || !out) { g_create_err = "null argument"; return KG_ERR_ARG; }
    int rc = check_params(params, g_create_err);
    if (rc) return rc;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        g_create_err = std::string("no CUDA device: ") + cudaGetErrorString(e);
        return KG_ERR_CUDA;
    }
    if (device >= 0) {
        e = cudaSetDevice(device);
        if (e != cudaSuccess) { g_create_err = cudaGetErrorString(e); return KG_ERR_CUDA; }
    }
    kg_handle* h = new kg_handle();
    h->prm = *params;
    cudaGetDevice(&h->device);
    e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { g_create_err = cudaGetErrorString(e); delete h; return KG_ERR_CUDA; }
    int lo_prio = 0, hi_prio = 0;
    cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio);
    e = cudaStreamCreateWithPriority(&h->aux, cudaStreamNonBlocking, hi_prio);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming);
    if (e != cudaSuccess) { g_create_err = cudaGetErrorString(e); cudaStreamDestroy(h->stream); delete h; return KG_ERR_CUDA; }
    e = cudaMallocHost(&h->h_res, sizeof(double) * MAX_SLOTS * RES_STRIDE);
    if (e == cudaSuccess) e = cudaMallocHost(&h->h_status, sizeof(int) * MAX_SLOTS);
    if (e != cudaSuccess) {
        g_create_err = cudaGetErrorString(e);
        cudaEventDestroy(h->ev_fork); cudaEventDestroy(h->ev_join);
        cudaStreamDestroy(h->aux); cudaStreamDestroy(h->stream);
        delete h;
        return KG_ERR_NOMEM;
    }
    *out = h;
    return KG_OK;
}

}  // namespace

extern "C" {

int kg_create(const kg_params* params, int device, kg_handle** out) { return create_handle(params, device, out); }

int kg_destroy(kg_handle* h) {
    if (!h) return KG_ERR_ARG;
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
    cudaStreamSynchronize(h->aux);
    free_pools(h);
    release_pools(h->spare_pools);
    h->mdl.release();
    h->cur_dl = nullptr;
    h->dscratch.release();
    if (h->d_tri) cudaFree(h->d_tri);
    if (h->sv_buf) cudaFree(h->sv_buf);
    if (h->s_in) { cudaStreamSynchronize(h->s_in); cudaStreamDestroy(h->s_in); }
    if (h->s_out) { cudaStreamSynchronize(h->s_out); cudaStreamDestroy(h->s_out); }
    if (h->h_res) cudaFreeHost(h->h_res);
    if (h->h_status) cudaFreeHost(h->h_status);
    cudaEventDestroy(h->ev_fork);
    cudaEventDestroy(h->ev_join);
    cudaStreamDestroy(h->aux);
    cudaStreamDestroy(h->stream);
    delete h;
    return KG_OK;
}

int kg_topology_footprint(const kg_params* params, const kg_topology* topo, int64_t* bytes) {
    if (!params || !topo || !bytes) return KG_ERR_ARG;
    Flat F;
    std::string err;
    int rc = flatten(*params, *topo, F, err);
    if (rc) { g_create_err = err; return rc; }
    *bytes = device_bytes(F, params->precision);
    return KG_OK;
}

int kg_upload_topology(kg_handle* h, const kg_topology* topo) {
    if (!h || !topo) return fail(h, KG_ERR_ARG, "null argument");
    if (h->is_batch) return fail(h, KG_ERR_STATE, "a batch handle admits problems with kg_batch_admit");
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
    release_pools(h->spare_pools);
    Flat F = std::move(h->spare);
    DevLayout dl;
    std::string err;
    int rc = build_layout(h, *topo, 0, F, dl, err);
    if (rc) { free_pools(h); return fail(h, rc, err); }
    if (!h->probs.empty()) h->spare = std::move(h->probs[0].F);
    if (F.max_inc > MAX_INC) { free_pools(h); return fail(h, KG_ERR_TOPOLOGY, "a cell has more face incidences than supported (" + std::to_string(F.max_inc) + ")"); }
    if ((rc = make_pools(h, F.foff.back(), F.n_data))) return rc;
    Problem& pb = h->probs[0];
    pb.F = std::move(F);
    pb.dl = dl;
    pb.fbase = 0; pb.fsize = pb.F.foff.back(); pb.dbase = 0; pb.dsize = pb.F.n_data;
    h->fslab.alloc(pb.fsize, &pb.fbase);
    h->dslab.alloc(pb.dsize, &pb.dbase);
    pb.pp = params_of(h->prm, 0.0);
    pb.live = false;   // becomes live with its state
    h->have_state = false;
    h->sdf_partial = false;
    h->dirty = true;
    return KG_OK;
}

int kg_upload_state(kg_handle* h, const double* f, const double* w, const double* prim) {
    if (!h || !f || !w || !prim) return fail(h, KG_ERR_ARG, "null argument");
    if (h->is_batch || h->probs.empty() || h->probs[0].F.n_data == 0) return fail(h, KG_ERR_STATE, "upload a topology first");
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
    Problem& pb = h->probs[0];
    if (!pb.live) {
        // first state for this topology: the slabs were reserved by kg_upload_topology
        pb.live = true;
        h->dirty = true;
    }
    int rc = upload_problem_state(h, 0, f, w, prim, 0);
    if (rc) return rc;
    h->have_state = true;
    h->sdf_partial = false;   // a fresh state's slopes are zero
    return KG_OK;
}

int kg_download_state(kg_handle* h, double* f, double* w, double* prim, double* qf, double* sdf) {
    if (!h) return KG_ERR_ARG;
    if (!h->have_state) return fail(h, KG_ERR_STATE, "no state on the device");
    cudaSetDevice(h->device);
    return download_problem(h, 0, f, w, prim, qf, sdf);
}

int kg_download_sw(kg_handle* h, double* sw) {
    if (!h) return KG_ERR_ARG;
    if (!sw) return fail(h, KG_ERR_ARG, "null argument");
    if (h->is_batch) return fail(h, KG_ERR_STATE, "a batch handle: use kg_batch_download_sw");
    if (!h->have_state) return fail(h, KG_ERR_STATE, "no state on the device");
    cudaSetDevice(h->device);
    return sync_point_rows(h, 0, sw, 0.0, nullptr);
}

int kg_criterion(kg_handle* h, double adapt_coeffi_ps, double* lohner) {
    if (!h) return KG_ERR_ARG;
    if (!lohner) return fail(h, KG_ERR_ARG, "null argument");
    if (h->is_batch) return fail(h, KG_ERR_STATE, "a batch handle: use kg_batch_criterion");
    if (!h->have_state) return fail(h, KG_ERR_STATE, "no state on the device");
    cudaSetDevice(h->device);
    return sync_point_rows(h, 0, nullptr, adapt_coeffi_ps, lohner);
}

int kg_adapt(kg_handle* h, const kg_topology* topo, const kg_adapt_src* src) {
    if (!h) return KG_ERR_ARG;
    if (!topo || !src) return fail(h, KG_ERR_ARG, "null argument");
    if (h->is_batch) return fail(h, KG_ERR_STATE, "a batch handle: use kg_batch_adapt");
    if (!h->have_state) return fail(h, KG_ERR_STATE, "no state on the device");
    cudaSetDevice(h->device);
    return adapt_problem(h, 0, topo, src);
}

int kg_vs_conserve(kg_handle* h, const uint8_t* cell_flags) {
    if (!h) return KG_ERR_ARG;
    if (!cell_flags) return fail(h, KG_ERR_ARG, "null argument");
    if (h->is_batch) return fail(h, KG_ERR_STATE, "a batch handle: use kg_batch_vs_conserve");
    if (!h->have_state) return fail(h, KG_ERR_STATE, "no state on the device");
    cudaSetDevice(h->device);
    return vs_conserve(h, 0, cell_flags);
}

int kg_download_restart(kg_handle* h, const int32_t* quad_index, int32_t n_quads, double* vs_df, double* ws) {
    if (!h) return KG_ERR_ARG;
    if (h->is_batch) return fail(h, KG_ERR_STATE, "a batch handle: use kg_batch_download_restart");
    if (!h->have_state) return fail(h, KG_ERR_STATE, "no state on the device");
    cudaSetDevice(h->device);
    return download_restart(h, 0, quad_index, n_quads, vs_df, ws);
}

int kg_upload_restart(kg_handle* h, const int32_t* quad_index, int32_t n_quads, const double* vs_df, const double* ws) {
    if (!h || !vs_df || !ws) return fail(h, KG_ERR_ARG, "null argument");
    if (h->is_batch || h->probs.empty() || h->probs[0].F.n_data == 0) return fail(h, KG_ERR_STATE, "upload a topology first");
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
    Problem& pb = h->probs[0];
    const bool was_live = pb.live;
    if (!pb.live) { pb.live = true; h->dirty = true; }
    int rc = upload_restart(h, 0, quad_index, n_quads, vs_df, ws, 0);
    if (rc) { if (!was_live) pb.live = false; return rc; }
    h->have_state = true;
    h->sdf_partial = false;   // restart() builds its PsData with zero slopes
    return KG_OK;
}

int kg_vs_flags(kg_handle* h, const kg_vs_config* cfg, uint8_t* flags, double* eta, double* vr) {
    if (!h) return KG_ERR_ARG;
    if (!cfg || !flags) return fail(h, KG_ERR_ARG, "null argument");
    if (h->is_batch) return fail(h, KG_ERR_STATE, "a batch handle: use kg_batch_vs_flags");
    if (!h->have_state) return fail(h, KG_ERR_STATE, "no state on the device");
    cudaSetDevice(h->device);
    return vs_flags(h, 0, cfg, flags, eta, vr);
}

int kg_step(kg_handle* h, double dt, int64_t step, int32_t nsteps, kg_step_report* report) {
    if (!h) return KG_ERR_ARG;
    if (!h->have_state) return fail(h, KG_ERR_STATE, "upload topology and state first");
    if (nsteps < 0 || !(dt > 0.0)) return fail(h, KG_ERR_ARG, "nsteps must be >= 0 and dt > 0");
    cudaSetDevice(h->device);
    Problem& pb = h->probs[0];
    if (pb.pp.dt != dt) {
        int rc = set_prob_dt(h, 0, dt);
        if (rc) return rc;
    }
    KG_CUDA(h, cudaMemcpyAsync(h->d_step, &step, sizeof(int64_t), cudaMemcpyHostToDevice, h->stream));
    double ms = 0.0;
    int64_t launches = 0;
    int rc = run_steps(h, nsteps, &ms, &launches);
    if (rc) return rc;
    kg_step_report r;
    fill_report(h, 0, ms, launches, &r);
    if (report) *report = r;
    if (r.status) return fail(h, r.status, r.status == KG_ERR_NONFINITE ? "non-finite primitive variables" : "rho <= 0 or lambda <= 0");
    return KG_OK;
}

int kg_serve(kg_handle* h, int32_t n_requests, const double* const* f_in, const double* const* w_in,
             const double* const* prim_in, double dt, int64_t step0, int32_t nsteps, double* const* f_out,
             double* const* w_out, double* const* prim_out, double* const* qf_out, kg_step_report* reports) {
    if (!h) return KG_ERR_ARG;
    if (h->is_batch || h->probs.empty() || h->probs[0].F.n_data == 0) return fail(h, KG_ERR_STATE, "upload a topology first");
    if (n_requests < 0 || nsteps < 0 || !(dt > 0.0)) return fail(h, KG_ERR_ARG, "n_requests and nsteps must be >= 0 and dt > 0");
    if (n_requests == 0) return KG_OK;
    if (!f_in || !w_in || !prim_in) return fail(h, KG_ERR_ARG, "null argument");
    for (int32_t r = 0; r < n_requests; ++r)
        if (!f_in[r] || !w_in[r] || !prim_in[r]) return fail(h, KG_ERR_ARG, "null input state");
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
    return serve(h, n_requests, f_in, w_in, prim_in, dt, step0, nsteps, f_out, w_out, prim_out, qf_out, reports);
}

int kg_profile_enable(kg_handle* h, int enable) {
    if (!h) return KG_ERR_ARG;
    h->prof = enable != 0;
    if (h->prof) { h->pnames.clear(); h->pms.clear(); h->pcount.clear(); h->punits.clear(); }
    return KG_OK;
}

int kg_profile_read(kg_handle* h, const char** names, double* total_ms, int64_t* launches, int32_t cap, int32_t* count) {
    if (!h || !count) return KG_ERR_ARG;
    h->pname_ptrs.clear();
    for (auto& s : h->pnames) h->pname_ptrs.push_back(s.c_str());
    int n = (int)std::min<size_t>(h->pnames.size(), (size_t)std::max(cap, 0));
    for (int i = 0; i < n; ++i) {
        if (names) names[i] = h->pname_ptrs[i];
        if (total_ms) total_ms[i] = h->pms[i];
        if (launches) launches[i] = h->pcount[i];
    }
    *count = (int32_t)h->pnames.size();
    return KG_OK;
}

int kg_profile_units(kg_handle* h, int64_t* units, int32_t cap, int32_t* count) {
    if (!h || !count) return KG_ERR_ARG;
    const int n = (int)std::min<size_t>(h->punits.size(), (size_t)std::max(cap, 0));
    for (int i = 0; i < n && units; ++i) units[i] = h->punits[i];
    *count = (int32_t)h->punits.size();
    return KG_OK;
}

int kg_memory_footprint(const kg_handle* h, int64_t* bytes) {
    if (!h || !bytes) return KG_ERR_ARG;
    *bytes = h->pool_bytes + h->topo_bytes;
    return KG_OK;
}

int kg_last_error(const kg_handle* h, char* buf, size_t cap) {
    if (!buf || cap == 0) return KG_ERR_ARG;
    std::snprintf(buf, cap, "%s", h ? h->err.c_str() : g_create_err.c_str());
    return KG_OK;
}

int kg_use_graph(kg_handle* h, int enable) {
    if (!h) return KG_ERR_ARG;
    h->use_graph = enable != 0;
    return KG_OK;
}

int kg_autotune(kg_handle* h, int enable) {
    if (!h) return KG_ERR_ARG;
    h->autotune = enable != 0;
    h->tuned_version = -1;
    if (!h->autotune) { h->sched = 0; h->sched_ctas = 0; }
    return KG_OK;
}

int kg_device_flatten(kg_handle* h, int enable) {
    if (!h) return KG_ERR_ARG;
    if (h->is_batch && h->devflat != (enable != 0))
        for (const Problem& pb : h->probs)
            if (pb.live) return fail(h, KG_ERR_STATE, "a batch's problems share one layout builder: set it before the first admission");
    h->devflat = enable != 0;
    return KG_OK;
}

int kg_layout_read(kg_handle* h, const char* name, void* out, int64_t cap, int64_t* bytes) {
    if (!h || !name || !bytes) return fail(h, KG_ERR_ARG, "null argument");
    cudaSetDevice(h->device);
    int rc = rebuild(h);
    if (rc) return rc;
    const Flat& M = h->M;
    const DevLayout* L = h->cur_dl;
    const Dev& P = h->dev;
    const void* ptr = nullptr;
    int64_t n = -1;
#define LAY(nm, field, count) if (!std::strcmp(name, nm)) { ptr = P.field; n = (int64_t)(count) * (int64_t)sizeof(*P.field); }
    LAY("slope_ops", slope_ops, L ? L->n_slope_ops : (int64_t)M.slope_ops.size());
    LAY("slope_nbr", slope_nbr, L ? L->n_slope_nbr : (int64_t)M.slope_nbr.size());
    LAY("cell_slope_op", cell_slope_op, L ? L->n_pass : (int64_t)M.cell_slope_op.size());
    LAY("pass_cells", pass_cells, L ? L->n_pass : (int64_t)M.pass_cells.size());
    LAY("screc", screc, L ? L->n_pass : (int64_t)M.screc.size());
    LAY("crit_ops", crit_ops, L ? L->n_crit_ops : (int64_t)M.crit_ops.size());
    LAY("crit_nbr", crit_nbr, L ? L->n_crit_nbr : (int64_t)M.crit_nbr.size());
    LAY("inc_off", inc_off, L ? L->n_fluid + 1 : (int64_t)M.inc_off.size());
    LAY("inc", inc, L ? L->n_inc : (int64_t)M.inc.size());
    LAY("bc_prim", bc_prim, L ? L->n_bc * MAXW : (int64_t)M.bc_prim.size());
    LAY("bc_hl", bc_hl, L ? L->n_bc * 2 * MAXW : (int64_t)M.bc_hl.size());
    LAY("fluid_cells", fluid_cells, L ? L->n_fluid : (int64_t)M.fluid_cells.size());
    LAY("fluid_reg", fluid_reg, L ? L->n_fluid : (int64_t)M.fluid_reg.size());
    LAY("fcrec", fcrec, L ? L->n_fluid : (int64_t)M.fcrec.size());
    LAY("regrec", regrec, L ? L->n_fluid : (int64_t)M.regrec.size());
    LAY("r2rec", r2rec, L ? L->n_fluid : (int64_t)M.r2rec.size());
    LAY("slope_items", slope_items, M.slope_items.size());
    LAY("p_off", p_off, M.p_off.size());
    LAY("p_j0", p_j0, M.p_j0.size());
    LAY("p_cnt", p_cnt, M.p_cnt.size());
    LAY("ib_nbr", ib_nbr, M.ib_nbr.size());
    LAY("wall_ops", wall_ops, M.wall_ops.size());
    LAY("solid_ops", solid_ops, M.solid_ops.size());
#undef LAY
    if (!std::strcmp(name, "reg_list")) { ptr = h->d_reg; n = (int64_t)h->n_reg * 4; }
    if (!std::strcmp(name, "nonreg_list")) { ptr = h->d_nonreg; n = (int64_t)h->n_nonreg * 4; }
    if (!std::strcmp(name, "r2_list")) { ptr = h->d_r2; n = (int64_t)h->n_r2 * 4; }
    if (!std::strcmp(name, "inner_list")) { ptr = h->d_inner; n = (int64_t)h->n_inner * 4; }
    if (!std::strcmp(name, "innerp_list")) { ptr = h->d_innerp; n = (int64_t)h->n_innerp * 4; }
    if (n < 0) return fail(h, KG_ERR_ARG, std::string("unknown layout array ") + name);
    *bytes = n;
    if (out && n > 0) {
        if (cap < n) return fail(h, KG_ERR_ARG, "output buffer too small");
        KG_CUDA(h, cudaMemcpyAsync(out, ptr, (size_t)n, cudaMemcpyDeviceToHost, h->stream));
        KG_CUDA(h, cudaStreamSynchronize(h->stream));
    }
    return KG_OK;
}

int kg_fuse_slopes(kg_handle* h, int enable) {
    if (!h) return KG_ERR_ARG;
    if (h->fuse_off == (enable == 0)) return KG_OK;
    cudaSetDevice(h->device);
    // the last step's slopes complete under the current layout before it changes
    int rc = complete_last_slopes(h);
    if (rc) return rc;
    h->fuse_off = enable == 0;
    h->dirty = true;
    return KG_OK;
}

int kg_autotune_result(const kg_handle* h, int32_t* schedule, int32_t* ctas_per_sm, double* trial_ms, int32_t cap) {
    if (!h) return KG_ERR_ARG;
    if (schedule) *schedule = h->sched;
    if (ctas_per_sm) *ctas_per_sm = h->sched_ctas;
    if (trial_ms) for (int i = 0; i < std::min(cap, 8); ++i) trial_ms[i] = h->tune_ms[i];
    return KG_OK;
}

// ---- batches -------------------------------------------------------------------
int kg_batch_create(const kg_params* params, int device, int64_t pool_bytes, kg_handle** out) {
    int rc = create_handle(params, device, out);
    if (rc) return rc;
    kg_handle* h = *out;
    h->is_batch = true;
    const int D = params->dim;
    size_t ss = params->precision == KG_PREC_FP64 ? 8 : 4;
    int64_t per_elem = (int64_t)ss * (2 + D) + (params->precision == KG_PREC_FP64 ? 0 : 8);
    int64_t fcap = pool_bytes / per_elem;
    int64_t dcap = std::max<int64_t>(4096, fcap / 64);
    fcap -= dcap * (int64_t)(sizeof(double) * (2 * MAXW + MAXD)) / per_elem;
    if (fcap <= 0) { kg_destroy(h); *out = nullptr; g_create_err = "pool too small"; return KG_ERR_BUDGET; }
    rc = make_pools(h, fcap, dcap);
    if (rc) { std::string m = h->err; kg_destroy(h); *out = nullptr; g_create_err = m; return rc; }
    return KG_OK;
}

int kg_batch_admit(kg_handle* h, const kg_params* params, const kg_topology* topo, const double* f, const double* w,
                   const double* prim, double dt, int64_t step, int32_t* slot) {
    if (!h || !params || !topo || !f || !w || !prim || !slot) return fail(h, KG_ERR_ARG, "null argument");
    if (!h->is_batch) return fail(h, KG_ERR_STATE, "not a batch handle");
    if (params->dim != h->prm.dim || params->ndf != h->prm.ndf || params->precision != h->prm.precision ||
        params->flux != h->prm.flux || params->marching != h->prm.marching)
        return fail(h, KG_ERR_ARG, "a batch holds problems of one dim / precision / flux / marching");
    if (!(dt > 0.0)) return fail(h, KG_ERR_ARG, "dt must be > 0");
    cudaSetDevice(h->device);
    int s = -1;
    for (int i = 0; i < MAX_SLOTS; ++i) if (!h->probs[i].live) { s = i; break; }
    if (s < 0) return fail(h, KG_ERR_BUDGET, "all problem slots are in use");
    cudaStreamSynchronize(h->stream);
    Flat F;
    DevLayout dl;
    std::string err;
    int rc = h->devflat ? device_flatten(*params, *topo, s, h->stream, F, dl, h->dscratch, err) : flatten(*params, *topo, F, err);
    if (rc) return fail(h, rc, err);
    if (F.max_inc > MAX_INC) return fail(h, KG_ERR_TOPOLOGY, "a cell has more face incidences than supported");
    rc = place_problem(h, s, std::move(F), *params, f, w, prim, dt, step);
    if (rc) return rc;
    h->probs[s].dl = dl;
    *slot = s;
    return KG_OK;
}

int kg_batch_release(kg_handle* h, int32_t slot) {
    if (h && h->is_batch) {
        // the last step's slopes of the lazy cells, while the layout still holds this problem
        cudaSetDevice(h->device);
        const int rc0 = complete_last_slopes(h);
        if (rc0) return rc0;
    }
    if (!h || !h->is_batch || slot < 0 || slot >= MAX_SLOTS || !h->probs[slot].live) return fail(h, KG_ERR_ARG, "bad slot");
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
    Problem& pb = h->probs[slot];
    h->fslab.release(pb.fbase, pb.fsize);
    h->dslab.release(pb.dbase, pb.dsize);
    pb = Problem();
    h->dirty = true;
    return KG_OK;
}

int kg_batch_step(kg_handle* h, int32_t nsteps, kg_step_report* reports, int32_t cap) {
    if (!h || !h->is_batch || nsteps < 0) return fail(h, KG_ERR_ARG, "bad argument");
    cudaSetDevice(h->device);
    double ms = 0.0;
    int64_t launches = 0;
    int rc = run_steps(h, nsteps, &ms, &launches);
    if (rc) return rc;
    int bad = 0;
    for (int s : h->live) {
        kg_step_report r;
        fill_report(h, s, ms, launches, &r);
        if (reports && s < cap) reports[s] = r;
        if (r.status) bad = r.status;
    }
    if (bad) return fail(h, bad, "a problem of the batch produced invalid primitive variables (see its report)");
    return KG_OK;
}

int kg_batch_download(kg_handle* h, int32_t slot, double* f, double* w, double* prim, double* qf) {
    if (!h || !h->is_batch || slot < 0 || slot >= MAX_SLOTS || !h->probs[slot].live) return fail(h, KG_ERR_ARG, "bad slot");
    cudaSetDevice(h->device);
    return download_problem(h, slot, f, w, prim, qf, nullptr);
}

int kg_batch_download_sw(kg_handle* h, int32_t slot, double* sw) {
    if (!h || !h->is_batch || slot < 0 || slot >= MAX_SLOTS || !h->probs[slot].live || !sw) return fail(h, KG_ERR_ARG, "bad slot");
    cudaSetDevice(h->device);
    return sync_point_rows(h, slot, sw, 0.0, nullptr);
}

int kg_batch_criterion(kg_handle* h, int32_t slot, double adapt_coeffi_ps, double* lohner) {
    if (!h || !h->is_batch || slot < 0 || slot >= MAX_SLOTS || !h->probs[slot].live || !lohner) return fail(h, KG_ERR_ARG, "bad slot");
    cudaSetDevice(h->device);
    return sync_point_rows(h, slot, nullptr, adapt_coeffi_ps, lohner);
}

int kg_batch_adapt(kg_handle* h, int32_t slot, const kg_topology* topo, const kg_adapt_src* src) {
    if (!h || !h->is_batch || slot < 0 || slot >= MAX_SLOTS || !h->probs[slot].live) return fail(h, KG_ERR_ARG, "bad slot");
    if (!topo || !src) return fail(h, KG_ERR_ARG, "null argument");
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
    return adapt_problem(h, slot, topo, src);
}

int kg_batch_download_restart(kg_handle* h, int32_t slot, const int32_t* quad_index, int32_t n_quads, double* vs_df, double* ws) {
    if (!h || !h->is_batch || slot < 0 || slot >= MAX_SLOTS || !h->probs[slot].live) return fail(h, KG_ERR_ARG, "bad slot");
    cudaSetDevice(h->device);
    return download_restart(h, slot, quad_index, n_quads, vs_df, ws);
}

int kg_batch_vs_conserve(kg_handle* h, int32_t slot, const uint8_t* cell_flags) {
    if (!h || !h->is_batch || slot < 0 || slot >= MAX_SLOTS || !h->probs[slot].live) return fail(h, KG_ERR_ARG, "bad slot");
    if (!cell_flags) return fail(h, KG_ERR_ARG, "null argument");
    cudaSetDevice(h->device);
    return vs_conserve(h, slot, cell_flags);
}

int kg_batch_vs_flags(kg_handle* h, int32_t slot, const kg_vs_config* cfg, uint8_t* flags, double* eta, double* vr) {
    if (!h || !h->is_batch || slot < 0 || slot >= MAX_SLOTS || !h->probs[slot].live) return fail(h, KG_ERR_ARG, "bad slot");
    if (!cfg || !flags) return fail(h, KG_ERR_ARG, "null argument");
    cudaSetDevice(h->device);
    return vs_flags(h, slot, cfg, flags, eta, vr);
}

int kg_batch_info(const kg_handle* h, int32_t* n_live, int64_t* f_free_elems, int64_t* bytes_per_elem) {
    if (!h || !h->is_batch) return KG_ERR_ARG;
    int n = 0;
    for (auto& p : h->probs) n += p.live ? 1 : 0;
    if (n_live) *n_live = n;
    if (f_free_elems) *f_free_elems = h->fslab.free_total();
    if (bytes_per_elem) *bytes_per_elem = (int64_t)storage_size(h) * (2 + h->prm.dim) + (h->prm.precision == KG_PREC_FP64 ? 0 : 8);
    return KG_OK;
}

int kg_batch_set_dt(kg_handle* h, int32_t slot, double dt) {
    if (!h || !h->is_batch || slot < 0 || slot >= MAX_SLOTS || !h->probs[slot].live || !(dt > 0.0)) return fail(h, KG_ERR_ARG, "bad argument");
    return set_prob_dt(h, slot, dt);
}

}  // extern "C"

// save_result's rows (IO/Output.jl:198-255): as save_result first runs update_slope! and
// update_solid_cell!, the slopes are recomputed from the current f and the solid cells updated
// (the state changes the reference makes too); save_boundary_result! then rebuilds each
// SolidNeighbor's wall distribution (refreshing its wall-direction slope, as the reference's
// boundary_slope! view does) without keeping it: the records' f blocks are restored after
// their rows are taken.
int kg_download_solution(kg_handle* h, const int32_t* quad_index, int32_t n_quads, double* ps_prim, double* ps_qf,
                         double* wall_rows) {
    if (!h) return KG_ERR_ARG;
    if (h->is_batch) return fail(h, KG_ERR_STATE, "a batch handle: save_result rows are per single-problem handle");
    if (!h->have_state) return fail(h, KG_ERR_STATE, "no state on the device");
    cudaSetDevice(h->device);
    int rc = rebuild(h);
    if (rc) return rc;
    Problem& pb = h->probs[0];
    const Flat& L = pb.F;
    if ((rc = check_quads(h, L, quad_index, n_quads))) return rc;
    const int D = h->prm.dim, NW = D + 2, NC = L.n_cells, NWALL = L.n_walls;
    const int WR = 2 * D + 2 + D * (D + 1) / 2;
    const Flat& M = h->M;
    Dev P = h->dev;
    P.f_in = h->parity == 0 ? h->fA : h->fB;
    P.f_out = h->parity == 0 ? h->fB : h->fA;
    cudaStream_t s = h->stream;
    cudaError_t e = enqueue_slopes_full(h, P, s);
    if (e == cudaSuccess && !M.solid_ops.empty())
        e = dispatch(h, [&](auto Lc) { return decltype(Lc)::solid(P, (int)M.solid_ops.size(), s); });
    if (e != cudaSuccess) return cuda_fail(h, e, "save_result: slopes and solid cells");
    if (wall_rows && NWALL > 0) {
        const size_t ss = storage_size(h);
        const int64_t w0 = pb.fbase + L.foff[NC], w1 = pb.fbase + L.foff[NC + NWALL];
        const size_t wb = (size_t)(w1 - w0) * ss;
        char* tmp = nullptr;
        e = cudaMalloc((void**)&tmp, 2 * wb + sizeof(double) * (size_t)NWALL * WR);
        if (e != cudaSuccess) return fail(h, KG_ERR_NOMEM, "cudaMalloc save_result rows");
        char* fa = (char*)P.f_in + (size_t)w0 * ss;
        char* fb = (char*)P.f_out + (size_t)w0 * ss;
        double* drows = (double*)(tmp + 2 * wb);
        e = cudaMemcpyAsync(tmp, fa, wb, cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(tmp + wb, fb, wb, cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess) e = dispatch(h, [&](auto Lc) { return decltype(Lc)::wall(P, (int)M.wall_ops.size(), M.max_nv, s); });
        if (e == cudaSuccess) e = dispatch(h, [&](auto Lc) { return decltype(Lc)::wall_rows(P, (int)M.wall_ops.size(), drows, s); });
        if (e == cudaSuccess) e = cudaMemcpyAsync(fa, tmp, wb, cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(fb, tmp + wb, wb, cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(wall_rows, drows, sizeof(double) * (size_t)NWALL * WR, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        cudaFree(tmp);
        if (e != cudaSuccess) return cuda_fail(h, e, "save_result: wall rows");
    }
    if (ps_prim || ps_qf) {
        std::vector<double> pp((size_t)NC * MAXW), qq((size_t)NC * MAXD);
        KG_CUDA(h, cudaMemcpyAsync(pp.data(), h->prim + pb.dbase * MAXW, sizeof(double) * pp.size(), cudaMemcpyDeviceToHost, s));
        KG_CUDA(h, cudaMemcpyAsync(qq.data(), h->qf + pb.dbase * MAXD, sizeof(double) * qq.size(), cudaMemcpyDeviceToHost, s));
        KG_CUDA(h, cudaStreamSynchronize(s));
        const double nan = std::numeric_limits<double>::quiet_NaN();
        if (ps_prim) std::fill(ps_prim, ps_prim + (size_t)n_quads * NW, nan);
        if (ps_qf) std::fill(ps_qf, ps_qf + (size_t)n_quads * D, nan);
        for (int c = 0; c < NC; ++c) {
            if (L.dbe[c] < 0) continue;   // PS_Solution of a solid cell: NaN (IO/Types.jl:56-63)
            const int64_t q = quad_index ? quad_index[c] : c;
            if (ps_prim) for (int e2 = 0; e2 < NW; ++e2) ps_prim[q * NW + e2] = pp[(size_t)c * MAXW + e2];
            if (ps_qf) for (int d = 0; d < D; ++d) ps_qf[q * D + d] = qq[(size_t)c * MAXD + d];
        }
    }
    return KG_OK;
}
