// tp_batch.cu — batching form: many independent simulations advanced by one CUDA-graph launch.
//
// A batch bundles handles (each one group of instances that share a cell grid, e.g. instances
// of one particle spacing placed side by side with gaps wider than the kernel support) with
// their device state.  tp_batch_capture records `steps` CarpenterKennedy2N54 steps of every
// member into one CUDA graph: the members are parallel branches (fork/join through events on
// one stream per member), each branch the member's fused integrator with list capacities fixed
// beforehand, so the graph contains no host synchronisation.  tp_batch_launch replays it on a
// caller stream.  tp_batch_autotune times trial steps of every member on scratch copies of its
// state over the pair pass (neighbour lists or, in the FP32 form, cell tiles staged in shared
// memory) x neighbour-list skins x pair-kernel block sizes and keeps the fastest combination.
//
// Persistent mode (tp_batch_set_mode(b, TP_BATCH_PERSISTENT), FP32 members on neighbour lists):
// the graph keeps the members' neighbour search, pack and Adami passes as parallel branches but
// joins them before every pair stage, which is one persistent launch for all members: about as
// many blocks as fit on the GPU take work items (a 256-slot tile of one member, the largest
// member first) from a counter until all members' slots are done.
#include <algorithm>
#include <cmath>
#include <new>
#include <string>
#include <vector>

#include "tp_api_internal.h"

struct tp_batch {
    struct Member {
        tp_handle* h = nullptr;
        double* v = nullptr;
        double* u = nullptr;
        double dt = 0.0;
        size_t nv = 0, nu = 0;  // element counts of v and u
        cudaStream_t stream = nullptr;
        cudaEvent_t join = nullptr;
        int pair_block = 128;
        double skin = 0.05;
        int pair_mode = TP_PAIR_GATHER;
        double trial_ms = 0.0;
    };
    std::vector<Member> m;
    cudaStream_t main = nullptr;
    cudaEvent_t fork = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long steps = 0;
    int mode = TP_BATCH_BRANCHES;
    unsigned* counter = nullptr;  // work-item counter of the persistent pair pass (device)
    std::string last_error;
};

namespace {

using namespace tp;

tp_status bfail(tp_batch* b, tp_status st, const std::string& msg) {
    if (b) b->last_error = msg;
    return st;
}

#define B_CUDA(b, call)                                                             \
    do {                                                                            \
        cudaError_t e_ = (call);                                                    \
        if (e_ != cudaSuccess)                                                      \
            return bfail(b, TP_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

tp_status member_fail(tp_batch* b, size_t k, tp_status st) {
    const char* e = tp_last_error(b->m[k].h);
    return bfail(b, st, "member " + std::to_string(k) + ": " + (e ? e : ""));
}

void drop_graph(tp_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    b->steps = 0;
}

// The members' stages interleaved around one persistent pair launch per stage (see the file
// comment); called between cudaStreamBeginCapture and cudaStreamEndCapture on b->main.
tp_status record_persistent(tp_batch* b, int64_t steps) {
    const size_t n = b->m.size();
    std::vector<size_t> order(n);
    for (size_t k = 0; k < n; ++k) order[k] = k;
    std::sort(order.begin(), order.end(), [&](size_t x, size_t y) {
        tp_config cx{}, cy{};
        tp_get_config(b->m[x].h, &cx);
        tp_get_config(b->m[y].h, &cy);
        return cx.n_fluid > cy.n_fluid;
    });
    tp_config c0{};
    tp_get_config(b->m[0].h, &c0);
    B_CUDA(b, cudaEventRecord(b->fork, b->main));
    std::vector<char> capturing(n, 0);
    for (size_t k = 0; k < n; ++k) {
        tp_batch::Member& mb = b->m[k];
        B_CUDA(b, cudaStreamWaitEvent(mb.stream, b->fork, 0));
        bool cap = false;
        tp_status st = integrator_begin(mb.h, mb.v, mb.u, steps, &cap);
        if (st != TP_OK) return member_fail(b, k, st);
        capturing[k] = cap;
    }
    bool std_cfg = true;
    for (int64_t step = 0; step < steps; ++step) {
        for (int stage = 0; stage < 5; ++stage) {
            for (size_t k = 0; k < n; ++k) {
                tp_batch::Member& mb = b->m[k];
                tp_status st = integrator_stage_pre(mb.h, step, stage);
                if (st != TP_OK) return member_fail(b, k, st);
                B_CUDA(b, cudaEventRecord(mb.join, mb.stream));
                B_CUDA(b, cudaStreamWaitEvent(b->main, mb.join, 0));
            }
            Pair32Batch B{};
            B.n = (int)n;
            int tiles = 0;
            for (size_t r = 0; r < n; ++r) {
                const size_t k = order[r];
                tp_status st = integrator_stage_pair(b->m[k].h, stage, b->m[k].dt, &B.m[r],
                                                     step == steps - 1 && stage == 4);
                if (st != TP_OK) return member_fail(b, k, st);
                B.tile0[r] = tiles;
                tiles += (B.m[r].nf + kBatchTile - 1) / kBatchTile;
                std_cfg = std_cfg && fp32_batch_pair_std(B.m[r].P);
            }
            B.tile0[n] = tiles;
            if (fp32_batch_pair(B, c0.ndims, std_cfg, b->counter, b->main) != TP_OK)
                return bfail(b, TP_ERR_CUDA, "tp_batch_capture: persistent pair launch failed");
            B_CUDA(b, cudaEventRecord(b->fork, b->main));
            for (size_t k = 0; k < n; ++k) {
                tp_batch::Member& mb = b->m[k];
                B_CUDA(b, cudaStreamWaitEvent(mb.stream, b->fork, 0));
                tp_status st = integrator_stage_post(mb.h);
                if (st != TP_OK) return member_fail(b, k, st);
            }
        }
    }
    for (size_t k = 0; k < n; ++k) {
        tp_batch::Member& mb = b->m[k];
        tp_status st = integrator_end(mb.h, mb.v, mb.u, capturing[k] != 0);
        if (st != TP_OK) return member_fail(b, k, st);
        B_CUDA(b, cudaEventRecord(mb.join, mb.stream));
        B_CUDA(b, cudaStreamWaitEvent(b->main, mb.join, 0));
    }
    return TP_OK;
}

// Persistent mode needs FP32 members on neighbour lists with one ndims and one model setup.
tp_status check_persistent(tp_batch* b) {
    if (b->m.size() > (size_t)kBatchMaxMembers)
        return bfail(b, TP_ERR_UNSUPPORTED, "persistent mode: at most " +
                                                std::to_string(kBatchMaxMembers) + " members");
    tp_config c0{};
    tp_get_config(b->m[0].h, &c0);
    for (size_t k = 0; k < b->m.size(); ++k) {
        tp_config c{};
        tp_get_config(b->m[k].h, &c);
        if (c.precision != TP_PRECISION_FP32 || b->m[k].h->pair_mode != TP_PAIR_GATHER)
            return bfail(b, TP_ERR_UNSUPPORTED,
                         "persistent mode: every member must be an FP32 handle on neighbour lists");
        if (c.ndims != c0.ndims || c.viscosity_model != c0.viscosity_model ||
            c.density_diffusion_model != c0.density_diffusion_model ||
            (c.viscosity_beta == 0.0) != (c0.viscosity_beta == 0.0))
            return bfail(b, TP_ERR_UNSUPPORTED,
                         "persistent mode: members must share ndims and the model switches");
    }
    return TP_OK;
}

// Scratch copies of a member's state (autotuning and warm-up never touch the caller's state).
struct Scratch {
    double* v = nullptr;
    double* u = nullptr;
    ~Scratch() {
        if (v) cudaFree(v);
        if (u) cudaFree(u);
    }
};

tp_status make_scratch(tp_batch* b, const tp_batch::Member& mb, Scratch& s) {
    B_CUDA(b, cudaMalloc((void**)&s.v, mb.nv * sizeof(double)));
    B_CUDA(b, cudaMalloc((void**)&s.u, mb.nu * sizeof(double)));
    B_CUDA(b, cudaMemcpyAsync(s.v, mb.v, mb.nv * sizeof(double), cudaMemcpyDeviceToDevice,
                              mb.stream));
    B_CUDA(b, cudaMemcpyAsync(s.u, mb.u, mb.nu * sizeof(double), cudaMemcpyDeviceToDevice,
                              mb.stream));
    return TP_OK;
}

tp_status restore_scratch(tp_batch* b, const tp_batch::Member& mb, Scratch& s) {
    B_CUDA(b, cudaMemcpyAsync(s.v, mb.v, mb.nv * sizeof(double), cudaMemcpyDeviceToDevice,
                              mb.stream));
    B_CUDA(b, cudaMemcpyAsync(s.u, mb.u, mb.nu * sizeof(double), cudaMemcpyDeviceToDevice,
                              mb.stream));
    return TP_OK;
}

}  // namespace

extern "C" {

tp_status tp_batch_create(tp_handle* const* handles, int32_t n, tp_batch** out) {
    if (!out || !handles || n <= 0) return TP_ERR_ARGUMENT;
    *out = nullptr;
    tp_batch* b = new (std::nothrow) tp_batch();
    if (!b) return TP_ERR_CUDA;
    b->m.resize((size_t)n);
    for (int k = 0; k < n; ++k) {
        if (!handles[k]) {
            delete b;
            return TP_ERR_ARGUMENT;
        }
        b->m[k].h = handles[k];
    }
    cudaError_t e = cudaStreamCreateWithFlags(&b->main, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->counter, sizeof(unsigned));
    for (auto& mb : b->m) {
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&mb.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&mb.join, cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        tp_batch_destroy(b);
        return TP_ERR_CUDA;
    }
    *out = b;
    return TP_OK;
}

tp_status tp_batch_destroy(tp_batch* b) {
    if (!b) return TP_OK;
    if (b->main) cudaStreamSynchronize(b->main);
    drop_graph(b);
    for (auto& mb : b->m) {
        if (mb.stream) {
            cudaStreamSynchronize(mb.stream);
            tp_set_stream(mb.h, nullptr);  // the handle outlives the batch's streams
            cudaStreamDestroy(mb.stream);
        }
        if (mb.join) cudaEventDestroy(mb.join);
    }
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->main) cudaStreamDestroy(b->main);
    if (b->counter) cudaFree(b->counter);
    delete b;
    return TP_OK;
}

tp_status tp_batch_set_state(tp_batch* b, int32_t k, double* v_ode, double* u_ode, double dt) {
    if (!b) return TP_ERR_ARGUMENT;
    if (k < 0 || k >= (int32_t)b->m.size() || !v_ode || !u_ode || !(dt > 0.0) ||
        !std::isfinite(dt))
        return bfail(b, TP_ERR_ARGUMENT, "tp_batch_set_state: bad member, array or dt");
    tp_batch::Member& mb = b->m[(size_t)k];
    tp_config c;
    tp_status st = tp_get_config(mb.h, &c);
    if (st != TP_OK) return member_fail(b, (size_t)k, st);
    mb.v = v_ode;
    mb.u = u_ode;
    mb.dt = dt;
    mb.nv = (size_t)c.n_fluid * (size_t)(c.ndims + 1);
    mb.nu = (size_t)c.n_fluid * (size_t)c.ndims;
    drop_graph(b);
    return TP_OK;
}

tp_status tp_batch_autotune(tp_batch* b, int32_t trial_steps, int32_t* pair_block_out,
                            double* skin_out, int32_t* pair_mode_out, double* ms_out) {
    if (!b) return TP_ERR_ARGUMENT;
    if (trial_steps <= 0) return bfail(b, TP_ERR_ARGUMENT, "tp_batch_autotune: trial_steps <= 0");
    static const int kBlocks[3] = {64, 128, 256};
    static const double kSkins[4] = {0.03, 0.05, 0.1, 0.2};
    drop_graph(b);
    cudaEvent_t e0, e1;
    B_CUDA(b, cudaEventCreate(&e0));
    B_CUDA(b, cudaEventCreate(&e1));
    tp_status result = TP_OK;
    for (size_t k = 0; k < b->m.size() && result == TP_OK; ++k) {
        tp_batch::Member& mb = b->m[k];
        if (!mb.v) {
            result = bfail(b, TP_ERR_NOT_READY, "tp_batch_autotune: member without state");
            break;
        }
        Scratch s;
        result = make_scratch(b, mb, s);
        if (result != TP_OK) break;
        tp_status st = tp_set_stream(mb.h, mb.stream);
        double best = INFINITY;
        tp_config cfg{};
        if (st == TP_OK) st = tp_get_config(mb.h, &cfg);
        // the tiled pass exists in the FP32 form only and launches fixed 256-thread blocks
        const int last_mode = cfg.precision == TP_PRECISION_FP32 ? TP_PAIR_TILED : TP_PAIR_GATHER;
        for (int mode = TP_PAIR_GATHER; mode <= last_mode; ++mode) {
          if (mode == TP_PAIR_SYMMETRIC) continue;
          if (st == TP_OK) st = tp_set_pair_mode(mb.h, mode);
          for (double skin : kSkins) {
            if (st == TP_OK) st = tp_set_skin(mb.h, skin);
            if (st == TP_OK) st = tp_prepare_lists(mb.h, s.u, 1.5);
            for (int blk : kBlocks) {
                if (st != TP_OK) break;
                if (mode == TP_PAIR_TILED && blk != 256) continue;
                st = tp_set_launch(mb.h, blk);
                if (st == TP_OK) result = restore_scratch(b, mb, s);
                if (st == TP_OK && result == TP_OK)
                    st = tp_integrate_ck2n54(mb.h, s.v, s.u, 0.0, mb.dt, 1);  // warm
                if (st != TP_OK || result != TP_OK) break;
                cudaEventRecord(e0, mb.stream);
                st = tp_integrate_ck2n54(mb.h, s.v, s.u, 0.0, mb.dt, trial_steps);
                cudaEventRecord(e1, mb.stream);
                if (st != TP_OK) break;
                cudaError_t ce = cudaEventSynchronize(e1);
                if (ce != cudaSuccess) {
                    result = bfail(b, TP_ERR_CUDA, cudaGetErrorString(ce));
                    break;
                }
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, e0, e1);
                const double per = (double)ms / trial_steps;
                if (per < best) {
                    best = per;
                    mb.pair_block = blk;
                    mb.skin = skin;
                    mb.pair_mode = mode;
                }
            }
            if (st != TP_OK || result != TP_OK) break;
          }
          if (st != TP_OK || result != TP_OK) break;
        }
        if (st == TP_OK) st = tp_sync(mb.h);
        if (st == TP_OK) st = tp_set_pair_mode(mb.h, mb.pair_mode);
        if (st == TP_OK) st = tp_set_skin(mb.h, mb.skin);
        if (st == TP_OK) st = tp_set_launch(mb.h, mb.pair_block);
        if (st != TP_OK && result == TP_OK) result = member_fail(b, k, st);
        mb.trial_ms = best;
        if (pair_block_out) pair_block_out[k] = mb.pair_block;
        if (skin_out) skin_out[k] = mb.skin;
        if (pair_mode_out) pair_mode_out[k] = mb.pair_mode;
        if (ms_out) ms_out[k] = best;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return result;
}

tp_status tp_batch_capture(tp_batch* b, int64_t steps, double growth) {
    if (!b) return TP_ERR_ARGUMENT;
    if (steps <= 0) return bfail(b, TP_ERR_ARGUMENT, "tp_batch_capture: steps <= 0");
    drop_graph(b);
    if (b->mode == TP_BATCH_PERSISTENT) {
        tp_status pr = check_persistent(b);
        if (pr != TP_OK) return pr;
    }
    // fixed list capacities, integrator state and a warm-up step (on scratch) per member
    for (size_t k = 0; k < b->m.size(); ++k) {
        tp_batch::Member& mb = b->m[k];
        if (!mb.v) return bfail(b, TP_ERR_NOT_READY, "tp_batch_capture: member without state");
        tp_status st = tp_set_stream(mb.h, mb.stream);
        if (st == TP_OK) st = tp_prepare_lists(mb.h, mb.u, growth);
        if (st != TP_OK) return member_fail(b, k, st);
        Scratch s;
        tp_status r = make_scratch(b, mb, s);
        if (r != TP_OK) return r;
        st = tp_integrate_ck2n54(mb.h, s.v, s.u, 0.0, mb.dt, 1);
        if (st == TP_OK) st = tp_sync(mb.h);
        if (st != TP_OK) return member_fail(b, k, st);
    }
    B_CUDA(b, cudaDeviceSynchronize());
    if (b->mode == TP_BATCH_PERSISTENT) {
        B_CUDA(b, cudaStreamBeginCapture(b->main, cudaStreamCaptureModeThreadLocal));
        tp_status pr = record_persistent(b, steps);
        cudaGraph_t g = nullptr;
        cudaError_t ee = cudaStreamEndCapture(b->main, &g);
        if (pr != TP_OK || ee != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            if (pr != TP_OK) return pr;
            return bfail(b, TP_ERR_CUDA, std::string("tp_batch_capture: ") +
                                             cudaGetErrorString(ee));
        }
        b->graph = g;
        B_CUDA(b, cudaGraphInstantiate(&b->exec, b->graph, 0));
        b->steps = steps;
        return TP_OK;
    }
    B_CUDA(b, cudaStreamBeginCapture(b->main, cudaStreamCaptureModeThreadLocal));
    tp_status result = TP_OK;
    cudaError_t ce = cudaEventRecord(b->fork, b->main);
    for (size_t k = 0; k < b->m.size() && ce == cudaSuccess && result == TP_OK; ++k) {
        tp_batch::Member& mb = b->m[k];
        ce = cudaStreamWaitEvent(mb.stream, b->fork, 0);
        if (ce != cudaSuccess) break;
        tp_status st = tp_integrate_ck2n54(mb.h, mb.v, mb.u, 0.0, mb.dt, steps);
        if (st != TP_OK) {
            result = member_fail(b, k, st);
            break;
        }
        ce = cudaEventRecord(mb.join, mb.stream);
        if (ce == cudaSuccess) ce = cudaStreamWaitEvent(b->main, mb.join, 0);
    }
    cudaGraph_t g = nullptr;
    cudaError_t ee = cudaStreamEndCapture(b->main, &g);
    if (result != TP_OK || ce != cudaSuccess || ee != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        if (result != TP_OK) return result;
        return bfail(b, TP_ERR_CUDA, std::string("tp_batch_capture: ") +
                                         cudaGetErrorString(ce != cudaSuccess ? ce : ee));
    }
    b->graph = g;
    B_CUDA(b, cudaGraphInstantiate(&b->exec, b->graph, 0));
    b->steps = steps;
    return TP_OK;
}

tp_status tp_batch_launch(tp_batch* b, void* stream) {
    if (!b) return TP_ERR_ARGUMENT;
    if (!b->exec) return bfail(b, TP_ERR_NOT_READY, "tp_batch_launch: nothing captured");
    B_CUDA(b, cudaGraphLaunch(b->exec, (cudaStream_t)stream));
    return TP_OK;
}

tp_status tp_batch_sync(tp_batch* b) {
    if (!b) return TP_ERR_ARGUMENT;
    B_CUDA(b, cudaDeviceSynchronize());
    for (size_t k = 0; k < b->m.size(); ++k) {
        tp_status st = tp_sync(b->m[k].h);
        if (st != TP_OK) return member_fail(b, k, st);
    }
    return TP_OK;
}

int64_t tp_batch_steps(const tp_batch* b) { return b ? (int64_t)b->steps : 0; }

tp_status tp_batch_set_mode(tp_batch* b, int32_t mode) {
    if (!b) return TP_ERR_ARGUMENT;
    if (mode != TP_BATCH_BRANCHES && mode != TP_BATCH_PERSISTENT)
        return bfail(b, TP_ERR_ARGUMENT,
                     "tp_batch_set_mode: mode must be TP_BATCH_BRANCHES or TP_BATCH_PERSISTENT");
    if (mode != b->mode) drop_graph(b);
    b->mode = mode;
    return TP_OK;
}

const char* tp_batch_last_error(const tp_batch* b) {
    return b ? b->last_error.c_str() : "null batch";
}

}  // extern "C"
