// Drives every C ABI entry point through create -> wall -> masses -> kick/drift/integrate ->
// diagnostics -> destroy, in both precision forms and in 2D and 3D (host logic only).
#include <cstdio>
#include <vector>

#include "tp_wcsph.h"

static int run(int nd, int precision) {
    tp_config c;
    tp_config_default(&c);
    c.ndims = nd;
    c.precision = precision;
    c.n_fluid = 3000;
    c.n_wall = 1500;
    c.smoothing_length = 0.035;
    c.sound_speed = 62.6;
    for (int d = 0; d < nd; ++d) {
        c.min_corner[d] = -0.05;
        c.max_corner[d] = 1.0;
    }
    c.acceleration[1] = -9.81;
    c.wall_clip_negative_pressure = 1;
    tp_handle* h = nullptr;
    int bad = 0;
    bad |= tp_create(&c, &h) != TP_OK;
    if (!h) return 1;
    std::vector<double> xw(c.n_wall * nd, 0.1), mw(c.n_wall, 0.4), mf(c.n_fluid, 0.4);
    std::vector<double> v(c.n_fluid * (nd + 1), 1000.0), u(c.n_fluid * nd, 0.5);
    std::vector<double> dv(v.size()), du(u.size()), pf(c.n_fluid), pw(c.n_wall);
    std::vector<int> cell(c.n_fluid), order(c.n_fluid), nff(c.n_fluid), nfw(c.n_fluid),
        nwf(c.n_wall);
    bad |= tp_kick(h, dv.data(), v.data(), u.data(), 0.0) != TP_ERR_NOT_READY;
    bad |= tp_set_wall(h, xw.data(), mw.data()) != TP_OK;
    bad |= tp_set_fluid_mass(h, mf.data()) != TP_OK;
    bad |= tp_enable_timing(h, 1) != TP_OK;
    bad |= tp_kick(h, dv.data(), v.data(), u.data(), 0.0) != TP_OK;
    bad |= tp_drift(h, du.data(), v.data(), u.data(), 0.0) != TP_OK;
    bad |= tp_set_skin(h, 0.2) != TP_OK;
    bad |= tp_set_launch(h, 256) != TP_OK;
    bad |= tp_set_launch(h, 100) != TP_ERR_ARGUMENT;
    bad |= tp_set_pair_mode(h, 5) != TP_ERR_ARGUMENT;
    bad |= tp_set_pair_mode(h, precision == 0 ? TP_PAIR_TILED : TP_PAIR_SYMMETRIC) !=
           TP_ERR_ARGUMENT;
    bad |= tp_set_pair_mode(h, precision == 0 ? TP_PAIR_SYMMETRIC : TP_PAIR_TILED) != TP_OK;
    bad |= tp_prepare_lists(h, u.data(), 1.5) != TP_OK;
    bad |= tp_integrate_ck2n54(h, v.data(), u.data(), 0.0, 1e-4, 2) != TP_OK;
    bad |= tp_integrate_ck2n54(h, v.data(), u.data(), 0.0, 1e-4, 1) != TP_OK;
    bad |= tp_kick(h, dv.data(), v.data(), u.data(), 0.0) != TP_OK;
    {
        int64_t rebuilds = -1;
        bad |= tp_rebuild_count(h, &rebuilds) != TP_OK || rebuilds < 0;
        bad |= tp_rebuild_count(h, nullptr) != TP_ERR_ARGUMENT;
    }
    bad |= tp_fluid_pressure(h, pf.data()) != TP_OK;
    bad |= tp_wall_state(h, pw.data(), nullptr, nullptr) != TP_OK;
    bad |= tp_nhs_debug(h, u.data(), cell.data(), order.data(), nff.data(), nfw.data(),
                        nwf.data()) != TP_OK;
    bad |= tp_fluid_pressure(h, pf.data()) != TP_ERR_NOT_READY;  // reordered since the kick
    bad |= tp_integrate_ck2n54(h, v.data(), u.data(), 0.0, 1e-4, 1) != TP_OK;
    bad |= tp_fluid_pressure(h, pf.data()) != TP_OK;
    double cons[5];
    bad |= tp_conservation(h, v.data(), cons) != TP_OK;
    double ms[8];
    bad |= tp_phase_times(h, ms, 8) != 3;
    bad |= tp_sync(h) != TP_OK;
    bad |= tp_cell_sort_noalloc(&c, u.data(), c.n_fluid, cell.data(), order.data(), nullptr) !=
           TP_OK;
    bad |= tp_integrate_ck2n54(h, v.data(), u.data(), 0.0, 1e-4, -1) != TP_ERR_ARGUMENT;
    bad |= tp_integrate_spv(h, v.data(), u.data(), 0.0, 1e-4, 3) != TP_OK;
    {
        std::vector<int32_t> perm(c.n_fluid);
        bad |= tp_sort_particles(h, v.data(), u.data(), 1, perm.data()) != TP_OK;
        bad |= tp_sort_particles(h, v.data(), u.data(), 0, nullptr) != TP_OK;
    }
    bad |= tp_integrate_spv(h, v.data(), u.data(), 0.0, 1e-4, -2) != TP_ERR_ARGUMENT;
    // differentiation form: forward with checkpoints, two backward sweeps, argument checks
    double pbar[3];
    std::vector<double> vbar(v.size(), 0.5), ubar(u.size(), 0.25);
    bad |= tp_adjoint_backward(h, vbar.data(), ubar.data(), pbar) != TP_ERR_NOT_READY;
    bad |= tp_adjoint_forward(h, v.data(), u.data(), 1e-4, 7, 3) != TP_OK;
    bad |= tp_adjoint_backward(h, vbar.data(), ubar.data(), pbar) != TP_OK;
    bad |= tp_adjoint_backward(h, vbar.data(), ubar.data(), pbar) != TP_OK;
    bad |= tp_adjoint_forward(h, v.data(), u.data(), 1e-4, 2, 5) != TP_OK;
    bad |= tp_adjoint_backward(h, vbar.data(), ubar.data(), pbar) != TP_OK;
    bad |= tp_adjoint_forward(h, v.data(), u.data(), 1e-4, 0, 5) != TP_ERR_ARGUMENT;
    bad |= tp_adjoint_forward(h, v.data(), u.data(), -1e-4, 3, 5) != TP_ERR_ARGUMENT;
    bad |= tp_adjoint_kernel_launches(h) <= 0;
    // diagnostics: pair distance and div_fast argument checks
    {
        std::vector<double> d2(5, 1.0), r(5);
        bad |= tp_pair_distance(h, d2.data(), r.data(), 5) != TP_OK;
        bad |= tp_pair_distance(h, nullptr, r.data(), 5) != TP_ERR_ARGUMENT;
        bad |= tp_pair_distance(h, d2.data(), r.data(), -1) != TP_ERR_ARGUMENT;
        bad |= tp_pair_distance(h, nullptr, nullptr, 0) != TP_OK;
    }
    // interpolation: with and without walls, argument checks
    {
        const int64_t np = 7;
        std::vector<double> pts(np * nd, 0.5), cd(np), vel(np * nd), pr(np), de(np);
        std::vector<int32_t> cnt(np);
        bad |= tp_interpolate_points(h, v.data(), u.data(), pts.data(), np, 0.07, 1, 1, 1,
                                     cd.data(), vel.data(), pr.data(), de.data(),
                                     cnt.data()) != TP_OK;
        bad |= tp_interpolate_points(h, v.data(), u.data(), pts.data(), np, 0.035, 0, 0, 0,
                                     cd.data(), vel.data(), pr.data(), de.data(),
                                     cnt.data()) != TP_OK;
        bad |= tp_interpolate_points(h, v.data(), u.data(), pts.data(), np, -1.0, 0, 0, 0,
                                     cd.data(), vel.data(), pr.data(), de.data(),
                                     cnt.data()) != TP_ERR_ARGUMENT;
    }
    // batching form: one-member batch, autotune, capture, launch, sync
    tp_batch* b = nullptr;
    tp_handle* hs[1] = {h};
    bad |= tp_batch_create(hs, 1, &b) != TP_OK;
    bad |= tp_batch_launch(b, nullptr) != TP_ERR_NOT_READY;
    bad |= tp_batch_capture(b, 2, 1.5) != TP_ERR_NOT_READY;
    bad |= tp_batch_set_state(b, 1, v.data(), u.data(), 1e-4) != TP_ERR_ARGUMENT;
    bad |= tp_batch_set_state(b, 0, v.data(), u.data(), 1e-4) != TP_OK;
    int32_t blk = 0;
    double skin = 0.0, tms = 0.0;
    int32_t mode = -1;
    bad |= tp_batch_autotune(b, 2, &blk, &skin, &mode, &tms) != TP_OK || mode < 0;
    bad |= (blk != 64 && blk != 128 && blk != 256);
    bad |= tp_batch_capture(b, 3, 1.5) != TP_OK;
    bad |= tp_batch_steps(b) != 3;
    bad |= tp_batch_launch(b, nullptr) != TP_OK;
    bad |= tp_batch_launch(b, nullptr) != TP_OK;
    bad |= tp_batch_sync(b) != TP_OK;
    // persistent mode: FP32 members on neighbour lists only
    bad |= tp_batch_set_mode(b, 7) != TP_ERR_ARGUMENT;
    bad |= tp_batch_set_mode(b, TP_BATCH_PERSISTENT) != TP_OK;
    bad |= tp_batch_steps(b) != 0;  // a mode change drops the graph
    {
        const tp_status want = precision == TP_PRECISION_FP32 && mode == TP_PAIR_GATHER
                                   ? TP_OK
                                   : TP_ERR_UNSUPPORTED;
        bad |= tp_batch_capture(b, 2, 1.5) != want;
        if (want == TP_OK) {
            bad |= tp_batch_steps(b) != 2;
            bad |= tp_batch_launch(b, nullptr) != TP_OK;
            bad |= tp_batch_sync(b) != TP_OK;
        }
    }
    bad |= tp_batch_set_mode(b, TP_BATCH_BRANCHES) != TP_OK;
    bad |= tp_batch_capture(b, 1, 1.5) != TP_OK;
    bad |= tp_batch_destroy(b) != TP_OK;
    tp_config back;
    bad |= tp_get_config(h, &back) != TP_OK;
    bad |= back.n_fluid != c.n_fluid;
    bad |= tp_destroy(h) != TP_OK;
    std::printf("nd=%d precision=%d bad=%d\n", nd, precision, bad);
    return bad;
}

int main() {
    int bad = 0;
    for (int nd = 2; nd <= 3; ++nd)
        for (int p = 0; p <= 1; ++p) bad |= run(nd, p);
    return bad;
}
