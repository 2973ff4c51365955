// tp_api_internal.h — launchers shared between the translation units of the library.
#pragma once

#include <type_traits>

#include "tp_handle.h"

namespace tp {

// FP64 drop-in form (tp_fp64.cu)
void fp64_pack(tp_handle* h, const double* u, const double* v, const double* m,
               const PhysState* src, PhysState* dst, const unsigned* gate);
void fp64_pack_wall(tp_handle* h, const double* x, const double* m);
void fp64_pack_pos(tp_handle* h, const double* u);
void fp64_adami(tp_handle* h);
void fp64_pair_kick(tp_handle* h, double* dv);
void fp64_pair_stage(tp_handle* h, PhysState& st, double A, double B, double dt, int first);
void fp64_count(tp_handle* h, int* nnb_ff, int* nnb_fw, int* nnb_wf);
void div_fast_check(tp_handle* h, double x64, const double* y64, double* out64, float x32,
                    const float* y32, float* out32, long long n);
void pair_distance_check(tp_handle* h, const double* d2, double* r, long long n);

// FP32 precision form (tp_fp32.cu)
void fp32_pack(tp_handle* h, const double* u, const double* v, const double* m,
               const PhysState* src, PhysState* dst, const unsigned* gate,
               bool skip_in_place = false);
void fp32_init_wall_state(tp_handle* h);
void fp32_adami(tp_handle* h);
void fp32_pair_kick(tp_handle* h, double* dv);
// src: the stage's source state (read in place when the stage did not rebuild); st: destination.
// With `desc` the pass is not launched: desc receives what the batched persistent pass needs.
void fp32_pair_stage(tp_handle* h, const PhysState& src, PhysState& st, double A, double B,
                     double dt, int first, Pair32Member* desc = nullptr, bool fuse_next = false);
// The batched persistent FP32 pair pass over B's members (same ndims and model switches).
void fp32_scatter_pressure(tp_handle* h, const int* ids, double* p_fluid);
bool fp32_batch_pair_std(const Phys32& P);
tp_status fp32_batch_pair(const Pair32Batch& B, int nd, bool std_cfg, unsigned* counter,
                          cudaStream_t stream);

// The fused integrator in pieces (tp_api.cu): tp_integrate_ck2n54 is begin, then per stage
// pre / pair / post, then end; the batching form's persistent capture interleaves its members'
// stages around one pair launch.
tp_status integrator_begin(tp_handle* h, double* v_ode, double* u_ode, int64_t n_steps,
                           bool* capturing);
tp_status integrator_stage_pre(tp_handle* h, int64_t step, int stage);
tp_status integrator_stage_pair(tp_handle* h, int stage, double dt, Pair32Member* desc,
                                bool last_stage);
tp_status integrator_stage_post(tp_handle* h);
tp_status integrator_end(tp_handle* h, double* v_ode, double* u_ode, bool capturing);

// API layer services used by the differentiation form (tp_api.cu)
tp_status api_fail(tp_handle* h, tp_status st, const std::string& msg);
tp_status api_cuda_fail(tp_handle* h, cudaError_t e, const char* where);
// Cell sort of fluid coordinates u (caller order): f_key (caller order), f_start, f_perm
// (slot -> caller index), f_skey; `maxcell` (optional, device) receives the largest occupancy.
tp_status sort_fluid_cells(tp_handle* h, const double* u, int* maxcell);
extern const double kCK2N54_A[5];
extern const double kCK2N54_B[5];

// Interpolation at points (tp_interp.cu); fluid cell sort (and, with walls, the Adami pass) of
// the same state must precede it on the handle's stream.
void interp_launch(tp_handle* h, const double* v, const double* u, const double* pts,
                   long long np, double hi, int walls, int cut_off_bnd, int clip,
                   int wall_velocity, double* cd, double* vel, double* pres, double* dens,
                   int* count);

// Differentiation form (tp_adjoint.cu)
void adjoint_release(tp_handle* h);

}  // namespace tp
