// kg_api.cu -- the C-ABI of libkitgpu.so (include/kitgpu.h).
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include "kg_device.cuh"

namespace kg {
template <int D, int NDF, typename T> struct Launch {
    static cudaError_t slope(const Dev&, int, int, cudaStream_t);
    static cudaError_t solid(const Dev&, int, cudaStream_t);
    static cudaError_t wall(const Dev&, int, int, cudaStream_t);
    static cudaError_t flux(const Dev&, int, int, double, int64_t, int, cudaStream_t);
};
cudaError_t launch_residual(const double*, int, double*, cudaStream_t);
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
// SolidNeighbor df starts as a copy of the donor df (Immersed_boundary.jl:290-298)
template <typename T>
__global__ void init_walls(const WallOp* ops, const int64_t* foff, T* fa, T* fb) {
    const WallOp op = ops[blockIdx.x];
    const int64_t src = foff[op.donor], dst = foff[op.data];
    const int64_t n = foff[op.data + 1] - dst;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) { fa[dst + i] = fa[src + i]; fb[dst + i] = fa[src + i]; }
}

struct DBuf {
    void* p = nullptr;
    size_t n = 0;
};

}  // namespace

void kg::set_global_error(const std::string& msg) { g_create_err = msg; }

struct kg_handle {
    kg_params prm{};
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    Flat F;
    bool topo = false, state = false;
    // device buffers
    std::vector<void*> allocs;
    Dev dev{};
    void* fA = nullptr;
    void* fB = nullptr;
    int parity = 0;             // 0: f_in = fA
    double* staging = nullptr;  // FP64 staging for the mixed form
    double* res_out = nullptr;  // [2*MAXW + 1] residual sums of the last checked step (+ step)
    double* h_res = nullptr;    // pinned copy
    int* d_status = nullptr;
    int64_t bytes = 0;
    // profiling
    bool prof = false;
    std::vector<std::string> pnames;
    std::vector<double> pms;
    std::vector<int64_t> pcount;
    std::vector<const char*> pname_ptrs;
    // graph
    bool use_graph = false;
    cudaGraphExec_t gexec = nullptr;
    int g_nsteps = -1, g_parity = -1;
    int64_t g_step_mod = -1;
    double g_dt = 0.0;
    int64_t last_launches = 0;
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

template <typename V>
int upload(kg_handle* h, const std::vector<V>& v, const V** out) {
    size_t n = std::max<size_t>(v.size(), 1) * sizeof(V);
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, n);
    if (e != cudaSuccess) return fail(h, KG_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    h->allocs.push_back(p);
    h->bytes += (int64_t)n;
    if (!v.empty()) {
        e = cudaMemcpy(p, v.data(), v.size() * sizeof(V), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_fail(h, e, "cudaMemcpy topology");
    }
    *out = (const V*)p;
    return KG_OK;
}
int alloc(kg_handle* h, size_t n, void** out) {
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(n, 8));
    if (e != cudaSuccess) return fail(h, KG_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    e = cudaMemset(p, 0, std::max<size_t>(n, 8));
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaMemset");
    h->allocs.push_back(p);
    h->bytes += (int64_t)n;
    *out = p;
    return KG_OK;
}

void free_device(kg_handle* h) {
    if (h->gexec) { cudaGraphExecDestroy(h->gexec); h->gexec = nullptr; }
    for (void* p : h->allocs) cudaFree(p);
    h->allocs.clear();
    h->bytes = 0;
    h->topo = h->state = false;
    h->fA = h->fB = nullptr;
    h->g_nsteps = -1;
}

size_t storage_size(const kg_handle* h) { return h->prm.precision == KG_PREC_FP64 ? sizeof(double) : sizeof(float); }

int prof_slot(kg_handle* h, const char* name) {
    for (size_t i = 0; i < h->pnames.size(); ++i)
        if (h->pnames[i] == name) return (int)i;
    h->pnames.push_back(name);
    h->pms.push_back(0.0);
    h->pcount.push_back(0);
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

// One step on the handle's stream (graph-capturable: no host synchronisation).
int enqueue_step(kg_handle* h, double dt, int64_t host_step, bool timed, int64_t* launches) {
    Flat& F = h->F;
    Dev P = h->dev;
    P.f_in = h->parity == 0 ? h->fA : h->fB;
    P.f_out = h->parity == 0 ? h->fB : h->fA;
    cudaStream_t s = h->stream;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto begin = [&]() -> int {
        if (!timed) return 0;
        cudaEventCreate(&e0); cudaEventCreate(&e1);
        cudaEventRecord(e0, s);
        return 0;
    };
    auto end = [&](const char* name) {
        if (!timed) return;
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        int k = prof_slot(h, name);
        h->pms[k] += ms;
        h->pcount[k] += 1;
        cudaEventDestroy(e0); cudaEventDestroy(e1);
    };
    cudaError_t e;
    int npass = (int)F.pass_off.size() - 1;
    for (int p = 0; p < npass; ++p) {
        int base = F.pass_cells_off[p], n = F.pass_cells_off[p + 1] - base;
        if (n <= 0) continue;
        begin();
        e = dispatch(h, [&](auto L) { return decltype(L)::slope(P, base, n, s); });
        if (e != cudaSuccess) return cuda_fail(h, e, "slope_kernel");
        end("slope_kernel");
        ++*launches;
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
    begin();
    e = dispatch(h, [&](auto L) { return decltype(L)::flux(P, F.n_fluid, F.max_nv, dt, host_step, h->prm.st_check_interval, s); });
    if (e != cudaSuccess) return cuda_fail(h, e, "flux_collide_kernel");
    end("flux_collide_kernel");
    ++*launches;
    if (host_step % h->prm.st_check_interval == 0) {
        e = launch_residual(h->dev.cell_res, F.n_fluid, h->res_out, s);
        if (e != cudaSuccess) return cuda_fail(h, e, "residual_kernel");
        ++*launches;
    }
    h->parity ^= 1;
    return KG_OK;
}

}  // namespace

extern "C" {

int kg_create(const kg_params* params, int device, kg_handle** out) {
    if (!params || !out) { g_create_err = "null argument"; return KG_ERR_ARG; }
    if (!(params->dim == 2 && params->ndf == 2) && !(params->dim == 3 && params->ndf == 1)) {
        g_create_err = "supported forms: dim 2 / ndf 2 and dim 3 / ndf 1";
        return KG_ERR_ARG;
    }
    if (params->precision != KG_PREC_FP64 && params->precision != KG_PREC_MIXED) { g_create_err = "bad precision"; return KG_ERR_ARG; }
    if (params->flux != KG_FLUX_CAIDVM && params->flux != KG_FLUX_DVM) { g_create_err = "bad flux"; return KG_ERR_ARG; }
    if (params->marching != KG_MARCH_CAIDVM && params->marching != KG_MARCH_EULER) { g_create_err = "bad marching"; return KG_ERR_ARG; }
    if (params->st_check_interval <= 0) { g_create_err = "st_check_interval must be positive"; return KG_ERR_ARG; }
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
    e = cudaMallocHost(&h->h_res, sizeof(double) * (2 * MAXW + 2));
    if (e != cudaSuccess) { g_create_err = cudaGetErrorString(e); cudaStreamDestroy(h->stream); delete h; return KG_ERR_NOMEM; }
    *out = h;
    return KG_OK;
}

int kg_destroy(kg_handle* h) {
    if (!h) return KG_ERR_ARG;
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
    free_device(h);
    if (h->h_res) cudaFreeHost(h->h_res);
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
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
    free_device(h);
    std::string err;
    int rc = flatten(h->prm, *topo, h->F, err);
    if (rc) return fail(h, rc, err);
    Flat& F = h->F;
    if (F.max_inc > MAX_INC) return fail(h, KG_ERR_TOPOLOGY, "a cell has more face incidences than supported (" + std::to_string(F.max_inc) + ")");
    size_t smax = (size_t)F.ndf * F.max_nv * sizeof(double);
    int dev_smem = 0;
    cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device);
    if (smax + 16384 > (size_t)dev_smem) return fail(h, KG_ERR_TOPOLOGY, "velocity grid too large for one CTA's shared memory");
    Dev& P = h->dev;
    P = Dev{};
    P.dim = F.dim; P.ndf = F.ndf; P.n_cells = F.n_cells; P.n_walls = F.n_walls;
    P.PG = (int64_t)F.vw.size();
#define UP(field, vec) do { int r__ = upload(h, F.vec, &P.field); if (r__) return r__; } while (0)
    UP(g_off, g_off); UP(vlev, vlev); UP(vw, vw); UP(vu, vu);
    UP(vuf, vuf); UP(vwf, vwf); UP(ax_off, ax_off); UP(ax_val, ax_val); UP(vidx, vidx);
    P.max_axis = F.max_axis;
    UP(foff, foff); UP(dgrid, dgrid); UP(dbe, dbe); UP(dmid, dmid); UP(dds, dds);
    UP(p_off, p_off); UP(p_j0, p_j0); UP(p_cnt, p_cnt);
    UP(slope_ops, slope_ops); UP(pass_cells, pass_cells); UP(cell_slope_op, cell_slope_op); UP(slope_nbr, slope_nbr);
    UP(fluid_cells, fluid_cells); UP(inc_off, inc_off); UP(inc, inc); UP(bc_prim, bc_prim);
    UP(solid_ops, solid_ops); UP(wall_ops, wall_ops); UP(ib_nbr, ib_nbr); UP(ib_dx, ib_dx);
    UP(cut_idx, cut_idx); UP(cut_gw, cut_gw); UP(cut_sw, cut_sw); UP(cvcw, cvcw);
#undef UP
    P.gamma = h->prm.gamma; P.K = h->prm.K; P.Pr = h->prm.Pr; P.omega = h->prm.omega; P.mu_ref = h->prm.mu_ref;
    P.flux = h->prm.flux; P.marching = h->prm.marching;
    int64_t nf = F.foff.back();
    size_t ss = storage_size(h);
    void* p;
    if ((rc = alloc(h, nf * ss, &h->fA))) return rc;
    if ((rc = alloc(h, nf * ss, &h->fB))) return rc;
    if ((rc = alloc(h, nf * F.dim * ss, &P.sdf))) return rc;
    if ((rc = alloc(h, sizeof(double) * F.n_data * MAXW, &p))) return rc; P.w = (double*)p;
    if ((rc = alloc(h, sizeof(double) * F.n_data * MAXW, &p))) return rc; P.prim = (double*)p;
    if ((rc = alloc(h, sizeof(double) * F.n_data * MAXD, &p))) return rc; P.qf = (double*)p;
    if ((rc = alloc(h, sizeof(double) * F.n_fluid * 2 * MAXW, &p))) return rc; P.cell_res = (double*)p;
    if ((rc = alloc(h, sizeof(int), &p))) return rc; P.status = (int*)p; h->d_status = P.status;
    if ((rc = alloc(h, sizeof(double) * (2 * MAXW + 2), &p))) return rc; h->res_out = (double*)p;
    if (h->prm.precision != KG_PREC_FP64) { if ((rc = alloc(h, sizeof(double) * nf, &p))) return rc; h->staging = (double*)p; }
    else h->staging = nullptr;
    h->parity = 0;
    h->topo = true;
    return KG_OK;
}

int kg_upload_state(kg_handle* h, const double* f, const double* w, const double* prim) {
    if (!h || !f || !w || !prim) return fail(h, KG_ERR_ARG, "null argument");
    if (!h->topo) return fail(h, KG_ERR_STATE, "upload a topology first");
    cudaSetDevice(h->device);
    Flat& F = h->F;
    const int D = F.dim, NW = D + 2;
    int64_t nfc = F.foff[F.n_cells];   // cells' part of f (walls follow)
    void* fin = h->parity == 0 ? h->fA : h->fB;
    void* fout = h->parity == 0 ? h->fB : h->fA;
    if (h->prm.precision == KG_PREC_FP64) {
        KG_CUDA(h, cudaMemcpyAsync(fin, f, sizeof(double) * nfc, cudaMemcpyHostToDevice, h->stream));
        KG_CUDA(h, cudaMemcpyAsync(fout, fin, sizeof(double) * nfc, cudaMemcpyDeviceToDevice, h->stream));
    } else {
        KG_CUDA(h, cudaMemcpyAsync(h->staging, f, sizeof(double) * nfc, cudaMemcpyHostToDevice, h->stream));
        to_storage<float><<<1024, 256, 0, h->stream>>>(h->staging, (float*)fin, nfc);
        to_storage<float><<<1024, 256, 0, h->stream>>>(h->staging, (float*)fout, nfc);
        KG_CUDA(h, cudaGetLastError());
    }
    if (!F.wall_ops.empty()) {
        if (h->prm.precision == KG_PREC_FP64)
            init_walls<double><<<(int)F.wall_ops.size(), 256, 0, h->stream>>>(h->dev.wall_ops, h->dev.foff, (double*)fin, (double*)fout);
        else
            init_walls<float><<<(int)F.wall_ops.size(), 256, 0, h->stream>>>(h->dev.wall_ops, h->dev.foff, (float*)fin, (float*)fout);
        KG_CUDA(h, cudaGetLastError());
    }
    KG_CUDA(h, cudaMemsetAsync(h->dev.sdf, 0, storage_size(h) * F.foff.back() * D, h->stream));
    std::vector<double> pw((size_t)F.n_data * MAXW, 0.0), pp((size_t)F.n_data * MAXW, 0.0);
    for (int c = 0; c < F.n_cells; ++c)
        for (int e = 0; e < NW; ++e) { pw[(size_t)c * MAXW + e] = w[(size_t)c * NW + e]; pp[(size_t)c * MAXW + e] = prim[(size_t)c * NW + e]; }
    KG_CUDA(h, cudaMemcpyAsync(h->dev.w, pw.data(), sizeof(double) * pw.size(), cudaMemcpyHostToDevice, h->stream));
    KG_CUDA(h, cudaMemcpyAsync(h->dev.prim, pp.data(), sizeof(double) * pp.size(), cudaMemcpyHostToDevice, h->stream));
    KG_CUDA(h, cudaMemsetAsync(h->dev.qf, 0, sizeof(double) * F.n_data * MAXD, h->stream));
    KG_CUDA(h, cudaMemsetAsync(h->d_status, 0, sizeof(int), h->stream));
    KG_CUDA(h, cudaStreamSynchronize(h->stream));   // pw / pp are host temporaries
    h->state = true;
    return KG_OK;
}

int kg_download_state(kg_handle* h, double* f, double* w, double* prim, double* qf, double* sdf) {
    if (!h) return KG_ERR_ARG;
    if (!h->state) return fail(h, KG_ERR_STATE, "no state on the device");
    cudaSetDevice(h->device);
    Flat& F = h->F;
    const int D = F.dim, NW = D + 2;
    int64_t nfc = F.foff[F.n_cells];
    void* fin = h->parity == 0 ? h->fA : h->fB;
    if (f) {
        if (h->prm.precision == KG_PREC_FP64) {
            KG_CUDA(h, cudaMemcpyAsync(f, fin, sizeof(double) * nfc, cudaMemcpyDeviceToHost, h->stream));
        } else {
            from_storage<float><<<1024, 256, 0, h->stream>>>((const float*)fin, h->staging, nfc);
            KG_CUDA(h, cudaGetLastError());
            KG_CUDA(h, cudaMemcpyAsync(f, h->staging, sizeof(double) * nfc, cudaMemcpyDeviceToHost, h->stream));
        }
    }
    if (sdf) {
        int64_t ns = nfc * D;
        if (h->prm.precision == KG_PREC_FP64) {
            KG_CUDA(h, cudaMemcpyAsync(sdf, h->dev.sdf, sizeof(double) * ns, cudaMemcpyDeviceToHost, h->stream));
        } else {
            // staging holds nf doubles; convert the sdf in dim chunks of nfc
            for (int d = 0; d < D; ++d) {
                from_storage<float><<<1024, 256, 0, h->stream>>>((const float*)h->dev.sdf + (int64_t)d * nfc, h->staging, nfc);
                KG_CUDA(h, cudaGetLastError());
                KG_CUDA(h, cudaMemcpyAsync(sdf + (int64_t)d * nfc, h->staging, sizeof(double) * nfc, cudaMemcpyDeviceToHost, h->stream));
                KG_CUDA(h, cudaStreamSynchronize(h->stream));
            }
        }
    }
    std::vector<double> pw((size_t)F.n_data * MAXW), pp((size_t)F.n_data * MAXW), pq((size_t)F.n_data * MAXD);
    if (w) KG_CUDA(h, cudaMemcpyAsync(pw.data(), h->dev.w, sizeof(double) * pw.size(), cudaMemcpyDeviceToHost, h->stream));
    if (prim) KG_CUDA(h, cudaMemcpyAsync(pp.data(), h->dev.prim, sizeof(double) * pp.size(), cudaMemcpyDeviceToHost, h->stream));
    if (qf) KG_CUDA(h, cudaMemcpyAsync(pq.data(), h->dev.qf, sizeof(double) * pq.size(), cudaMemcpyDeviceToHost, h->stream));
    KG_CUDA(h, cudaStreamSynchronize(h->stream));
    for (int c = 0; c < F.n_cells; ++c) {
        for (int e = 0; e < NW; ++e) {
            if (w) w[(size_t)c * NW + e] = pw[(size_t)c * MAXW + e];
            if (prim) prim[(size_t)c * NW + e] = pp[(size_t)c * MAXW + e];
        }
        if (qf) for (int d = 0; d < D; ++d) qf[(size_t)c * D + d] = pq[(size_t)c * MAXD + d];
    }
    return KG_OK;
}

int kg_step(kg_handle* h, double dt, int64_t step, int32_t nsteps, kg_step_report* report) {
    if (!h) return KG_ERR_ARG;
    if (!h->state) return fail(h, KG_ERR_STATE, "upload topology and state first");
    if (nsteps < 0 || !(dt > 0.0)) return fail(h, KG_ERR_ARG, "nsteps must be >= 0 and dt > 0");
    cudaSetDevice(h->device);
    cudaEvent_t t0, t1;
    KG_CUDA(h, cudaEventCreate(&t0));
    KG_CUDA(h, cudaEventCreate(&t1));
    KG_CUDA(h, cudaEventRecord(t0, h->stream));
    int64_t launches = 0;
    int64_t last_check = -1;
    const int iv = h->prm.st_check_interval;
    bool graph_ok = h->use_graph && !h->prof;
    if (graph_ok) {
        // a graph covers nsteps steps from a given f parity with the residual cadence baked
        // in, so it is reused only when step % interval repeats as well
        bool reuse = h->gexec && h->g_nsteps == nsteps && h->g_dt == dt && h->g_parity == h->parity &&
                     h->g_step_mod == step % iv;
        if (!reuse) {
            if (h->gexec) { cudaGraphExecDestroy(h->gexec); h->gexec = nullptr; }
            int parity0 = h->parity;
            cudaGraph_t graph;
            KG_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
            int rc = KG_OK;
            int64_t l = 0;
            for (int s = 0; s < nsteps && rc == KG_OK; ++s) rc = enqueue_step(h, dt, step + s, false, &l);
            cudaError_t ce = cudaStreamEndCapture(h->stream, &graph);
            if (rc) return rc;
            if (ce != cudaSuccess) return cuda_fail(h, ce, "cudaStreamEndCapture");
            ce = cudaGraphInstantiate(&h->gexec, graph, 0);
            cudaGraphDestroy(graph);
            if (ce != cudaSuccess) return cuda_fail(h, ce, "cudaGraphInstantiate");
            h->g_nsteps = nsteps; h->g_dt = dt; h->g_parity = parity0; h->g_step_mod = step % iv;
            h->last_launches = l;
            h->parity = parity0;
        }
        KG_CUDA(h, cudaGraphLaunch(h->gexec, h->stream));
        launches = h->last_launches;
        if (nsteps % 2) h->parity ^= 1;
        for (int s = 0; s < nsteps; ++s) if ((step + s) % iv == 0) last_check = step + s;
    } else {
        for (int s = 0; s < nsteps; ++s) {
            int rc = enqueue_step(h, dt, step + s, h->prof, &launches);
            if (rc) return rc;
            if ((step + s) % iv == 0) last_check = step + s;
        }
    }
    KG_CUDA(h, cudaEventRecord(t1, h->stream));
    KG_CUDA(h, cudaMemcpyAsync(h->h_res, h->res_out, sizeof(double) * 2 * MAXW, cudaMemcpyDeviceToHost, h->stream));
    int st = 0;
    KG_CUDA(h, cudaMemcpyAsync(&h->h_res[2 * MAXW], h->d_status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    KG_CUDA(h, cudaStreamSynchronize(h->stream));
    std::memcpy(&st, &h->h_res[2 * MAXW], sizeof(int));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, t0, t1);
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    if (report) {
        std::memset(report, 0, sizeof(*report));
        report->checked = last_check >= 0;
        report->checked_step = last_check;
        for (int e = 0; e < 5; ++e) { report->sum_res[e] = h->h_res[e]; report->sum_avg[e] = h->h_res[MAXW + e]; }
        report->device_ms = ms;
        report->phase_cells = h->F.phase_cells;
        report->kernel_launches = (int32_t)launches;
        report->status = st ? ((st & ST_NONFINITE) ? KG_ERR_NONFINITE : KG_ERR_NEGATIVE) : KG_OK;
    }
    if (st) return fail(h, (st & ST_NONFINITE) ? KG_ERR_NONFINITE : KG_ERR_NEGATIVE,
                        (st & ST_NONFINITE) ? "non-finite primitive variables" : "rho <= 0 or lambda <= 0");
    return KG_OK;
}

int kg_profile_enable(kg_handle* h, int enable) {
    if (!h) return KG_ERR_ARG;
    h->prof = enable != 0;
    if (h->prof) { h->pnames.clear(); h->pms.clear(); h->pcount.clear(); }
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

int kg_memory_footprint(const kg_handle* h, int64_t* bytes) {
    if (!h || !bytes) return KG_ERR_ARG;
    *bytes = h->bytes;
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

}  // extern "C"
