// kg_devflat.h -- the gather form of one problem built on the device (kg_devflat.cu).
#pragma once
#include <cuda_runtime.h>
#include <memory>
#include "kg_internal.h"

namespace kg {

// The arrays of one problem's gather form that a step reads, built on the device in the
// merged form of a single problem at data base 0 and f base 0 (one allocation, shared by the
// copies of the problem that refer to it; freed with the last).
struct DevLayout {
    std::shared_ptr<void> arena;
    size_t bytes = 0;
    SlopeOp* slope_ops = nullptr;
    NbrRef* slope_nbr = nullptr;
    int32_t* cell_slope_op = nullptr;
    int32_t* pass_cells = nullptr;
    SlopeCell* screc = nullptr;
    CritOp* crit_ops = nullptr;
    int32_t* crit_nbr = nullptr;
    int32_t* inc_off = nullptr;
    Incidence* inc = nullptr;
    double* bc_prim = nullptr;
    float* bc_hl = nullptr;
    uint8_t* fluid_reg = nullptr;
    uint8_t* fluid_r2 = nullptr;
    FluxCell* fcrec = nullptr;
    RegRec* regrec = nullptr;
    R2Rec* r2rec = nullptr;
    int32_t* fluid_cells = nullptr;
    int32_t* dsc = nullptr;        // data item -> pass-cell entry (R2 pass)
    int32_t* dfl = nullptr;        // data item -> fluid-list entry (R2 pass)
    int64_t n_slope_ops = 0, n_slope_nbr = 0, n_pass = 0, n_crit_ops = 0, n_crit_nbr = 0;
    int64_t n_fluid = 0, n_inc = 0, n_bc = 0, n_data = 0;
    void release() { arena.reset(); bytes = 0; }
};

// Device and pinned host scratch of the builder, kept by a handle and grown on demand.
struct DevScratch {
    void* dev = nullptr;
    void* pin = nullptr;
    size_t dev_cap = 0, pin_cap = 0;
    void release();
};

// Builds the gather form of topology t for problem slot `slot` on stream s: the host part
// (flatten_head, flatten_checks, flatten_ib) into F, the rest into L; F.devlay is set.
// Returns KG_OK or an error code with the host builder's message.
// t_ms (optional, 4 entries): host wall time of the host part (checks, grids, data table,
// pairings, wall records), of packing and uploading the arrays, of the counting kernels and of
// the rest (fills, slope-pass order, records)
int device_flatten(const kg_params& prm, const kg_topology& t, int slot, cudaStream_t s, Flat& F, DevLayout& L,
                   DevScratch& S, std::string& err, double* t_ms = nullptr);

// One device-built problem of a batch and its offsets in the merged layout (the host merge's
// accumulators: data and f base, slope-neighbour, slope-op, criterion-neighbour, incidence,
// boundary-record, pairing, grid and velocity-cell counts before it), with its local pass
// offsets and the merged start of each of its passes.
struct MergeIn {
    const DevLayout* L = nullptr;
    int64_t fbase = 0, PGacc = 0;
    int32_t dbase = 0, snb = 0, sops = 0, cacc = 0, incacc = 0, bcacc = 0, pairacc = 0, Gacc = 0;
    std::vector<int32_t> pass_off;
    std::vector<int32_t> pass_base;
};

// The merged gather form of device-built problems in M, equal to the host merge of their
// host-built forms; foff, dnv: the merged data table (host arrays, n_data entries and one more
// for foff); npc_total: the merged pass-cell entries.
int device_merge(const std::vector<MergeIn>& parts, int64_t n_data, int64_t npc_total, const int64_t* foff,
                 const int32_t* dnv, int D, cudaStream_t s, DevLayout& M, DevScratch& S, std::string& err);

// The R2 records and flags of a device-built layout (slopes in the flux kernel; zeros unless
// fuse and 2D); the flags also into r2 (host).
int device_r2(const Flat& M, DevLayout& L, bool fuse, cudaStream_t s, std::vector<uint8_t>& r2, std::string& err);

}  // namespace kg
