// tp_handle.h — host-side handle of the WCSPH library (C ABI object behind tp_handle*).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "tp_internal.cuh"

namespace tp {

struct AdjointState;  // differentiation form (tp_adjoint.cu)

// Timed phases of one RHS evaluation (labels of the reference's TimerOutputs sections):
//   0 "update nhs" (cell keys, scan, scatter, rank + pack incl. the fluid EOS),
//   1 "compute boundary pressure" (Adami), 2 "system interaction" (pair kernel + fused update).
constexpr int kNumPhases = 3;

// Per-particle physical state of the integrator, one copy of a ping-pong pair.  Slot order
// (the cell-sorted order of the previous stage).  FP64 form: u/tu = (nd, n) doubles,
// v/tv = (nd+1, n) doubles.  FP32 form: u/tu doubles as above, v/tv = float4 per particle
// {vx, vy, vz, rho - rho0}.
struct PhysState {
    double* u = nullptr;
    double* tu = nullptr;
    void* v = nullptr;
    void* tv = nullptr;
    void* m = nullptr;  // double (FP64) or float (FP32)
    int* id = nullptr;  // original (caller) index of the particle in this slot
};

}  // namespace tp

struct tp_handle {
    tp_config cfg{};
    tp::GridDesc grid{};
    tp::Phys phys{};
    tp::Phys32 phys32{};
    cudaStream_t stream = nullptr;
    bool wall_set = false;
    bool mass_set = false;
    bool timing = false;
    std::string last_error;

    // ---- fluid neighbour search (n_fluid entries unless noted) ----
    int* f_key = nullptr;     // cell key of particle i (source order)
    int* f_tmp = nullptr;     // atomic scatter order
    int* f_perm = nullptr;    // slot -> source index
    int* f_skey = nullptr;    // slot -> cell key
    int* f_count = nullptr;   // ncells, kept zero between uses
    int* f_start = nullptr;   // ncells + 1
    int* f_cursor = nullptr;  // ncells
    int* scan_partial = nullptr;
    int scan_blocks = 0;

    // ---- fluid records (slot order) ----
    // f_test: {ox, oy, oz, w}: offsets in the reference cell (FP32 neighbour tests, both forms);
    // w = x cell index (FP64) or rho - rho0 (FP32, rewritten every stage)
    float4* f_test = nullptr;
    void* f_pos = nullptr;     // FP64 form / diagnostics: double4 {x, y, z, p}
    void* f_vel = nullptr;     // FP64: double4 {v, rho};  FP32: float4 {v, m / rho}
    void* f_aux = nullptr;     // FP64: double4 (see the pack);  FP32: float p
    // FP32 pair record, 32 bytes per slot (one 256-bit load per neighbour):
    // {ox, oy, oz, rho - rho0, vx, vy, vz, m / rho}
    void* f_rec = nullptr;
    // the other record buffer of the FP32 integrator: a pair stage writes the next stage's records
    // there (the in-place pack of a stage without a rebuild is then skipped) and the two swap
    void* f_rec2 = nullptr;
    bool rec_prev_fused = false;    // the previous pair stage wrote this stage's records
    bool rec_fuse_pending = false;  // this stage's pair pass writes the next stage's records

    // ---- fluid masses in caller order (FP64) ----
    double* m_f = nullptr;

    // ---- wall (static, slot order) ----
    int* w_key = nullptr;
    int* w_tmp = nullptr;
    int* w_perm = nullptr;   // slot -> caller index
    int* w_skey = nullptr;
    int* w_start = nullptr;  // ncells + 1
    void* w_pos = nullptr;    // double4 {x, y, z, m} (both forms)
    float4* w_test = nullptr; // {ox, oy, oz, w}: w = x cell (FP64) or m / rho (FP32, Adami)
    // FP64: double4 (see the Adami pass); FP32: float4 {p, rho - rho0, m, m / rho}
    void* w_state = nullptr;
    float* w_p32 = nullptr;   // FP32: wall pressure of the last Adami pass (dense, for gathers)
    double* w_vol = nullptr;

    // ---- neighbour lists (tp_lists.cuh): entry k of slot s at list_at(k, n, s), chunks of 8 ----
    unsigned* l_ff = nullptr;  // fluid -> fluid candidates
    unsigned* l_fw = nullptr;  // fluid -> wall
    unsigned* l_wf = nullptr;  // wall -> fluid (Adami)
    int* c_ff = nullptr;
    int* c_fw = nullptr;
    int* c_wf = nullptr;
    int cap_ff = 0, cap_fw = 0, cap_wf = 0;
    // FP64 form: the exact pair lists of the current stage (|x_a - x_b| <= 2h, self excluded),
    // filtered from l_ff / l_fw at the start of every pair pass; plain slot indices, same layout
    // (ec_ff / ec_fw: their counts, kept by the separate filter pass of the symmetric mode)
    int* e_ff = nullptr;
    int* e_fw = nullptr;
    int* e_wf = nullptr;  // the walls' exact fluid lists of the Adami pass (FP64 form)
    int* ec_ff = nullptr;
    int* ec_fw = nullptr;
    int ecap_ff = 0, ecap_fw = 0, ecap_wf = 0;
    // FP64 form, symmetric pair mode: per-slot accumulator {dv (3), drho} of the pair pass
    double* acc = nullptr;
    int pair_mode = 0;  // TP_PAIR_GATHER (default), TP_PAIR_SYMMETRIC (FP64), TP_PAIR_TILED (FP32)
    // list radius 2h (1 + skin); rebuild after skin * h displacement.  0.05 measured best on
    // GB300 in both forms, at rest and in a 3 m/s flow (shorter lists outweigh the rebuilds).
    double skin = 0.05;
    double* x_build = nullptr;  // fluid positions at the last rebuild (slot order)
    double* grid_org = nullptr;  // per-axis cell origins of the FP32 cell size (GridDesc::org)
    int num_sms = 1;             // multiprocessors of the device (fixed-grid launches)
    unsigned* tile_ctr = nullptr;  // TileQueue counters of the fluid and wall list builds (2 + 2)
    unsigned* gate = nullptr;   // {force, max squared displacement bits, squared threshold bits,
                                //  next stage's displacement bits, rebuilds let through}
    int* d_max = nullptr;       // scratch for the largest cell occupancy
    int maxcell_w = 0;          // largest wall cell occupancy (walls are static)
    bool lists_fixed = false;   // capacity fixed by tp_prepare_lists (no sizing sync per call)
    // Which path the cell list, slot order and skin lists currently belong to: 0 none (next
    // use rebuilds), 1 the kick! path (slots map to caller indices through f_perm), 2 the fused
    // integrator (slots map to caller indices through its state's id array).  The owner reuses
    // them across calls until a particle has moved more than skin * h.
    int lists_owner = 0;
    // How the slot records (f_pos / f_aux, pressure of the last right-hand side) map to caller
    // indices: 0 not at all (an unconditional sort replaced f_perm since), 1 through f_perm
    // (kick! path), 2 through the integrator's final state id array.
    int records_order = 0;
    int pair_block = 128;      // threads per block of the pair / Adami kernels (autotuned)

    // ---- integrator ping-pong state ----
    tp::PhysState st[2];
    int cur = 0;

    // ---- conservation reduction scratch ----
    double* red_partial = nullptr;
    int red_blocks = 0;

    // ---- device error word ----
    int* d_err = nullptr;
    int* h_err = nullptr;  // pinned

    // Phase timing: kNumPhases + 1 events per RHS evaluation from a pool, read back once at
    // the end of the call (no synchronisation inside the stage loop).
    std::vector<cudaEvent_t> evpool;
    size_t ev_used = 0;
    double phase_ms[tp::kNumPhases] = {};
    long long launches = 0;  // kernel launches issued on this handle

    // ---- SymplecticPositionVerlet scratch: k, v_half, u_half (caller order) ----
    double* spv = nullptr;

    // ---- differentiation form: checkpoints, tape and adjoint buffers (tp_adjoint.cu) ----
    tp::AdjointState* adj = nullptr;
};
