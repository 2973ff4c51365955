// tp_oracle.cpp — FP64 CPU ORACLE for the WCSPH right-hand side of TrixiParticles.jl.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker: tests/, __graft_entry__.smoke() and the
// CPU-baseline leg of bench.py may load it; the product library never links or calls it.
//
// It restates, in plain C++ with IEEE double arithmetic and no FMA contraction (build with
// -ffp-contract=off), the reference's Float64 CPU path for the supported system pair.  Every
// function cites the reference lines (paths relative to the TrixiParticles.jl tree) whose
// evaluation order it follows.  Third-party pieces that are not in the reference tree are
// restated from their published algorithm:
//   * PointNeighbors.jl 0.6.6 GridNeighborhoodSearch + FullGridCellList: cell size = search
//     radius = compact support 2h; cells aligned at the coordinate origin
//     (cell = floor(x / cell_size)); one padding layer of cells around the bounding box;
//     neighbour cells visited in CartesianIndices order (x fastest); particles of one cell
//     visited in ascending index order (the order of a freshly built or serially updated
//     list); a pair is visited when dot(x_a - x_b, x_a - x_b) <= search_radius^2.
//   * OrdinaryDiffEqLowStorageRK 3, CarpenterKennedy2N54(williamson_condition=false): the
//     five-stage fourth-order 2N-storage scheme of Carpenter & Kennedy (1994), NASA TM-109112,
//     solution 3, applied as  tmp = dt*k; u += B1*tmp;  then per stage i>=2:
//     tmp = A_i*tmp; tmp += dt*k; u += B_i*tmp  (muladd fused, as the @muladd of that package).
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>

#include "../include/tp_wcsph.h"
#include "dual.h"

namespace {

using orc::val;

constexpr double kPi = 3.141592653589793;  // Float64(pi)
constexpr double kEps = 2.220446049250313e-16;  // eps(Float64)

// ---------------------------------------------------------------------------------------
// Smoothing kernels (src/general/smoothing_kernels.jl)
// ---------------------------------------------------------------------------------------

// WendlandC2Kernel normalisation, smoothing_kernels.jl:450-455.
inline double wc2_norm(int nd, double h_inv) {
    if (nd == 2) return (7.0 / (4.0 * kPi)) * (h_inv * h_inv);
    return (21.0 / (16.0 * kPi)) * ((h_inv * h_inv) * h_inv);
}

// kernel_unsafe(::WendlandC2Kernel), smoothing_kernels.jl:436-441 (@fastpow: t^4 = (t*t)^2).
// T: double, or a dual number for forward-mode derivatives (dual.h); h is a constant.
template <class T>
inline T wc2_kernel_unsafe(int nd, T r, double h) {
    double h_inv = 1.0 / h;
    T q = r * h_inv;
    T t = 1.0 - q / 2.0;
    T t2 = t * t;
    T t4 = t2 * t2;
    return (wc2_norm(nd, h_inv) * t4) * (2.0 * q + 1.0);
}

// kernel(kernel, r, h), smoothing_kernels.jl:30-34: zero outside the compact support 2h.
template <class T>
inline T wc2_kernel(int nd, T r, double h) {
    return (r < 2.0 * h) ? wc2_kernel_unsafe(nd, r, h) : T(0.0);
}

// kernel_deriv_div_r_unsafe(::WendlandC2Kernel), smoothing_kernels.jl:443-448.
template <class T>
inline T wc2_deriv_div_r(int nd, T r, double h) {
    double h_inv = 1.0 / h;
    T q = r * h_inv;
    T t = 1.0 - q / 2.0;
    T t3 = (t * t) * t;
    return ((-5.0 * wc2_norm(nd, h_inv)) * t3) * (h_inv * h_inv);
}

// SchoenbergCubicSplineKernel (smoothing_kernels.jl:191-227), used by the viscosity KAT only.
inline double scs_norm(int nd, double h_inv) {
    if (nd == 2) return (10.0 / (kPi * 7.0)) * (h_inv * h_inv);
    return (1.0 / kPi) * ((h_inv * h_inv) * h_inv);
}
inline double scs_deriv_div_r(int nd, double r, double h) {
    double h_inv = 1.0 / h;
    double q = r * h_inv;
    double a = 2.0 - q;
    double b = 1.0 - q;
    double result = ((-3.0) * (a * a)) / 4.0 + (3.0 * (q < 1.0 ? 1.0 : 0.0)) * (b * b);
    double kd = (scs_norm(nd, h_inv) * result) * h_inv;
    return kd / r;
}

// ---------------------------------------------------------------------------------------
// StateEquationCole, state_equations.jl:117-139.
// ---------------------------------------------------------------------------------------
struct Eos {
    double rho0, c, gamma, p_bg;
    bool clip;
    double B() const { return (rho0 * (c * c)) / gamma; }
    template <class T>
    T pressure(T rho) const {
        using std::pow;
        using std::isnan;
        T p = B() * (pow(rho / rho0, gamma) - 1.0) + p_bg;
        if (clip) p = (isnan(p) || p > 0.0) ? p : T(0.0);  // max(0, p)
        return p;
    }
    template <class T>
    T inverse(T p) const {
        using std::pow;
        T tmp = (p - p_bg) / B() + 1.0;
        return rho0 * pow(tmp, 1.0 / gamma);
    }
};

template <class T>
inline T clip_nonneg(T p) {  // max(p, 0) with Julia's NaN / signed-zero rules
    using std::isnan;
    if (isnan(p)) return p;
    return (p > 0.0) ? p : T(0.0);
}

// ---------------------------------------------------------------------------------------
// Cell grid (PointNeighbors FullGridCellList restated; see header comment).
// ---------------------------------------------------------------------------------------
struct Grid {
    int nd = 0;
    double cs = 0.0;
    int64_t cmin[3] = {0, 0, 0};
    int64_t n[3] = {1, 1, 1};
    int64_t ncells = 0;
    bool init(const tp_config& cfg) {
        nd = cfg.ndims;
        cs = 2.0 * cfg.smoothing_length;
        ncells = 1;
        for (int d = 0; d < 3; ++d) {
            if (d < nd) {
                int64_t lo = (int64_t)std::floor(cfg.min_corner[d] / cs) - 1;
                int64_t hi = (int64_t)std::floor(cfg.max_corner[d] / cs) + 1;
                cmin[d] = lo;
                n[d] = hi - lo + 1;
            } else {
                cmin[d] = 0;
                n[d] = 1;
            }
            ncells *= n[d];
        }
        return ncells > 0 && ncells < (int64_t(1) << 31);
    }
    // Returns false when the point is outside the inner (unpadded) grid.
    bool cell_of(const double* x, int64_t c[3]) const {
        bool ok = true;
        for (int d = 0; d < 3; ++d) {
            if (d < nd) {
                double g = std::floor(x[d] / cs) - (double)cmin[d];
                if (!(g >= 1.0 && g <= (double)(n[d] - 2))) {
                    ok = false;
                    g = std::isnan(g) ? 1.0 : std::min(std::max(g, 1.0), (double)(n[d] - 2));
                }
                c[d] = (int64_t)g;
            } else {
                c[d] = 0;
            }
        }
        return ok;
    }
    int64_t key(const int64_t c[3]) const { return c[0] + n[0] * (c[1] + n[1] * c[2]); }
};

struct CellList {
    std::vector<int32_t> key;    // per particle
    std::vector<int32_t> order;  // sorted position -> particle
    std::vector<int64_t> start;  // ncells + 1
    bool ok = true;
    template <class T>
    void build(const Grid& g, const T* x, int64_t n) {
        key.assign(n, 0);
        ok = true;
        for (int64_t i = 0; i < n; ++i) {
            int64_t c[3];
            double xv[3] = {0.0, 0.0, 0.0};
            for (int d = 0; d < g.nd; ++d) xv[d] = val(x[i * g.nd + d]);
            if (!g.cell_of(xv, c)) ok = false;
            key[i] = (int32_t)g.key(c);
        }
        order.resize(n);
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(),
                         [&](int32_t a, int32_t b) { return key[a] < key[b]; });
        start.assign(g.ncells + 1, 0);
        for (int64_t i = 0; i < n; ++i) start[key[i] + 1]++;
        for (int64_t c = 0; c < g.ncells; ++c) start[c + 1] += start[c];
    }
};

// Visits the neighbours b (of a list over coordinates xb) of the point xa in PointNeighbors
// order; f(b, pos_diff, distance) for every b with |xa - xb|^2 <= sr^2 (decided on the values).
template <class TA, class TB, class F>
inline void foreach_neighbor(const Grid& g, const CellList& cl, const TB* xb, const TA* xa,
                             double sr, F&& f) {
    using std::sqrt;
    using T = decltype(xa[0] - xb[0]);
    int64_t c[3];
    double xav[3] = {0.0, 0.0, 0.0};
    for (int d = 0; d < g.nd; ++d) xav[d] = val(xa[d]);
    g.cell_of(xav, c);
    const int nd = g.nd;
    const double sr2 = sr * sr;
    int64_t zlo = (nd == 3) ? c[2] - 1 : 0, zhi = (nd == 3) ? c[2] + 1 : 0;
    for (int64_t cz = zlo; cz <= zhi; ++cz)
        for (int64_t cy = c[1] - 1; cy <= c[1] + 1; ++cy)
            for (int64_t cx = c[0] - 1; cx <= c[0] + 1; ++cx) {
                int64_t k = cx + g.n[0] * (cy + g.n[1] * cz);
                for (int64_t s = cl.start[k]; s < cl.start[k + 1]; ++s) {
                    int32_t b = cl.order[s];
                    T pd[3] = {T(0.0), T(0.0), T(0.0)};
                    for (int d = 0; d < nd; ++d) pd[d] = xa[d] - xb[b * nd + d];
                    T d2 = pd[0] * pd[0] + pd[1] * pd[1];
                    if (nd == 3) d2 = d2 + pd[2] * pd[2];
                    if (val(d2) <= sr2) f(b, pd, sqrt(d2));
                }
            }
}

template <class TA, class TB>
inline auto dot(int nd, const TA* a, const TB* b) -> decltype(a[0] * b[0]) {
    auto s = a[0] * b[0] + a[1] * b[1];
    if (nd == 3) s = s + a[2] * b[2];
    return s;
}

// T = double: the oracle.  T = orc::Dual<N>: the same arithmetic carrying N directional
// derivatives (forward mode); masses and wall positions are constants, the state and the
// parameters alpha, delta and gravity are differentiable.
template <class T>
struct ModelT {
    tp_config cfg;
    Grid grid;
    Eos eos_f, eos_w;
    int nd;
    int64_t nf, nw;
    std::vector<double> xw, mw, mf;
    CellList wall_cl;
    // Per-kick outputs.
    std::vector<T> pf, pw, rhow, volw;
    CellList fluid_cl;
    bool grid_ok = true;
    // Monaghan alpha, Molteni-Colagrossi delta, gravity (the configuration's values)
    T alpha_p, delta_p, grav[3];

    bool init(const tp_config& c) {
        cfg = c;
        nd = c.ndims;
        nf = c.n_fluid;
        nw = c.n_wall;
        if (!grid.init(c)) return false;
        eos_f = {c.reference_density, c.sound_speed, c.exponent, c.background_pressure,
                 c.fluid_clip_negative_pressure != 0};
        eos_w = eos_f;
        eos_w.clip = false;
        pf.assign(nf, T(0.0));
        pw.assign(nw, T(0.0));
        rhow.assign(nw, T(c.reference_density));
        volw.assign(nw, T(0.0));
        alpha_p = c.viscosity_alpha;
        delta_p = c.density_diffusion_delta;
        for (int d = 0; d < 3; ++d) grav[d] = c.acceleration[d];
        return true;
    }

    // compute_pressure! (weakly_compressible_sph/system.jl:426-438).
    void fluid_pressure(const T* v) {
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < nf; ++i) pf[i] = eos_f.pressure(v[i * (nd + 1) + nd]);
    }

    // compute_pressure!(::AdamiPressureExtrapolation) (dummy_particles.jl:489-569) with the
    // gather boundary_pressure_extrapolation!(Val(true)) and boundary_pressure_inner!
    // (dummy_particles.jl:586-606, 637-672).
    void adami(const T* v, const T* u) {
        const double h = cfg.smoothing_length;
        const double sr = 2.0 * h;  // compact_support(wall, fluid) = model's 2h
        const T* g = grav;
#pragma omp parallel for schedule(dynamic, 64)
        for (int64_t w = 0; w < nw; ++w) {
            T P = 0.0, V = 0.0;
            foreach_neighbor(grid, fluid_cl, u, &xw[w * nd], sr,
                             [&](int32_t f, const T* pd, T r) {
                                 T rho_f = v[f * (nd + 1) + nd];
                                 T p_f = pf[f];
                                 T ra[3] = {g[0] - 0.0, g[1] - 0.0, g[2] - 0.0};
                                 T rpd[3] = {rho_f * pd[0], rho_f * pd[1],
                                             nd == 3 ? rho_f * pd[2] : T(0.0)};
                                 T hp = dot(nd, ra, rpd);
                                 T sum = ((cfg.pressure_offset + p_f) + 0.0) + hp;
                                 T W = wc2_kernel(nd, r, h);
                                 P += sum * W;
                                 V += W;
                             });
            if (V > kEps) P = P / V;
            if (cfg.wall_clip_negative_pressure) P = clip_nonneg(P);
            pw[w] = P;
            volw[w] = V;
            rhow[w] = eos_w.inverse(P);
        }
    }

    // kick! (semidiscretization.jl:589-612) for the fluid system; the wall contributes no
    // ODE rows (wall_boundary/system.jl:78-90).
    void kick(T* dv, const T* v, const T* u) {
        const double h = cfg.smoothing_length;
        const double sr = 2.0 * h;
        const double sr2 = sr * sr;
        // almostzero = sqrt(eps(compact_support^2)), rhs.jl:27-28; eps(x) = ulp spacing at x.
        const double almostzero = std::sqrt(std::nextafter(sr2, INFINITY) - sr2);
        const double c = cfg.sound_speed;
        const T alpha = alpha_p, delta = delta_p;
        const double beta = cfg.viscosity_beta, epsv = cfg.viscosity_epsilon;
        const bool visc = cfg.viscosity_model == TP_VISCOSITY_MONAGHAN;
        const bool diff = cfg.density_diffusion_model == TP_DIFFUSION_MOLTENI_COLAGROSSI;
        const int nv = nd + 1;

        // set_zero!(dv_ode), :600
        std::fill(dv, dv + nf * nv, T(0.0));
        // update_nhs!, neighborhood_search.jl:479-519
        fluid_cl.build(grid, u, nf);
        grid_ok = fluid_cl.ok && wall_cl.ok;
        // update_pressure! then update_boundary_interpolation!, :616-651
        fluid_pressure(v);
        adami(v, u);

        // system_interaction!: (fluid, fluid) then (fluid, wall), rhs.jl:5-127
#pragma omp parallel for schedule(dynamic, 64)
        for (int64_t a = 0; a < nf; ++a) {
            const T* xa = u + a * nd;
            const T* va = v + a * nv;
            const T rho_a = va[nd];
            const T p_a = pf[a];
            // ---- fluid-fluid ----
            T dva[3] = {T(0.0), T(0.0), T(0.0)}, drho = 0.0;
            foreach_neighbor(grid, fluid_cl, u, xa, sr, [&](int32_t b, const T* pd, T r) {
                if (r < almostzero) return;
                T s = wc2_deriv_div_r(nd, r, h);
                T grad[3] = {s * pd[0], s * pd[1], nd == 3 ? s * pd[2] : T(0.0)};
                const double m_b = mf[b];
                const T* vb = v + b * nv;
                const T rho_b = vb[nd];
                const T p_b = pf[b];
                // pressure_acceleration_continuity_density, pressure_acceleration.jl:34-41
                T coef = (-m_b) * ((p_a + p_b) / (rho_a * rho_b));
                for (int d = 0; d < nd; ++d) dva[d] = dva[d] + coef * grad[d];
                T vd[3] = {va[0] - vb[0], va[1] - vb[1], nd == 3 ? va[2] - vb[2] : T(0.0)};
                // ArtificialViscosityMonaghan, viscosity.jl:99-132
                if (visc) {
                    T vr = dot(nd, vd, pd);
                    if (vr < 0.0) {
                        double hh = (h + h) / 2.0;
                        T rho_mean = (rho_a + rho_b) / 2.0;
                        T mu = (hh * vr) / (r * r + epsv * (hh * hh));
                        T num = ((m_b * alpha) * c) * mu + (m_b * beta) * (mu * mu);
                        T f = num / rho_mean;
                        for (int d = 0; d < nd; ++d) dva[d] = dva[d] + f * grad[d];
                    }
                }
                // continuity_equation!, fluid.jl:179-197
                drho = drho + ((rho_a / rho_b) * m_b) * dot(nd, vd, grad);
                // density_diffusion! Molteni-Colagrossi, density_diffusion.jl:49-55, 213-240
                if (diff) {
                    T volume_b = m_b / rho_b;
                    T pc = (2.0 * (rho_a - rho_b)) / (r * r);
                    T psi[3] = {pc * pd[0], pc * pd[1], nd == 3 ? pc * pd[2] : T(0.0)};
                    T term = volume_b * dot(nd, psi, grad);
                    double havg = (h + h) / 2.0;
                    drho = drho + ((delta * havg) * c) * term;
                }
            });
            for (int d = 0; d < nd; ++d) dv[a * nv + d] = dv[a * nv + d] + dva[d];
            dv[a * nv + nd] = dv[a * nv + nd] + drho;
            // ---- fluid-wall ----
            T dvw[3] = {T(0.0), T(0.0), T(0.0)}, drhow = 0.0;
            foreach_neighbor(grid, wall_cl, xw.data(), xa, sr,
                             [&](int32_t b, const T* pd, T r) {
                                 if (r < almostzero) return;
                                 T s = wc2_deriv_div_r(nd, r, h);
                                 T grad[3] = {s * pd[0], s * pd[1], nd == 3 ? s * pd[2] : T(0.0)};
                                 const double m_b = mw[b];
                                 const T rho_b = rhow[b];
                                 const T p_b = pw[b];
                                 T coef = (-m_b) * ((p_a + p_b) / (rho_a * rho_b));
                                 for (int d = 0; d < nd; ++d) dvw[d] = dvw[d] + coef * grad[d];
                                 T vd[3] = {va[0] - 0.0, va[1] - 0.0,
                                            nd == 3 ? va[2] - 0.0 : T(0.0)};
                                 drhow = drhow + ((rho_a / rho_b) * m_b) * dot(nd, vd, grad);
                             });
            for (int d = 0; d < nd; ++d) dv[a * nv + d] = dv[a * nv + d] + dvw[d];
            dv[a * nv + nd] = dv[a * nv + nd] + drhow;
            // add_source_terms! -> add_acceleration!, semidiscretization.jl:701-731
            for (int d = 0; d < nd; ++d) dv[a * nv + d] = dv[a * nv + d] + grav[d];
        }
    }

    // interpolate_points (src/general/interpolation.jl:480-697) after the system update the
    // PostprocessCallback performs (update_systems_and_nhs, semidiscretization.jl:616-646:
    // fluid pressure from the current density, Adami wall state).  The neighbourhood searches
    // are copies with search radius = compact support 2 h_i (process_neighborhood_searches,
    // :492-534), i.e. cells of size 2 h_i; neighbours are visited system by system (fluid, then
    // wall) in that grid's order.  Outputs per point: computed_density, velocity (nd), pressure,
    // density, neighbor_count.
    void interpolate(const double* v, const double* u, const double* pts, int64_t np,
                     double hi, bool cut_off_bnd, bool clip, bool wall_velocity, double* cd,
                     double* vel, double* pres, double* dens, int32_t* count) {
        fluid_cl.build(grid, u, nf);
        fluid_pressure(v);
        adami(v, u);
        tp_config c2 = cfg;
        c2.smoothing_length = hi;  // Grid::init takes cell size 2 * smoothing_length
        Grid gi;
        gi.init(c2);
        CellList fcl, wcl;
        fcl.build(gi, u, nf);
        const bool walls = cut_off_bnd || wall_velocity;
        if (walls) wcl.build(gi, xw.data(), nw);
        const double sr = 2.0 * hi;
#pragma omp parallel for schedule(dynamic, 16)
        for (int64_t i = 0; i < np; ++i) {
            const double* x = pts + i * nd;
            double rho_c = 0.0, other = 0.0, shep = 0.0, shep_w = 0.0;
            double vv[3] = {0, 0, 0}, pp = 0.0, dd = 0.0;
            int32_t cnt = 0;
            foreach_neighbor(gi, fcl, u, x, sr, [&](int32_t b, const double*, double r) {
                const double m_b = mf[b];
                const double rho_b = v[b * (nd + 1) + nd];
                const double vol = m_b / rho_b;
                const double W = wc2_kernel(nd, r, hi);
                if (wall_velocity) shep_w += vol * W;
                rho_c += m_b * W;
                shep += vol * W;
                for (int d = 0; d < nd; ++d) vv[d] += (v[b * (nd + 1) + d] * vol) * W;
                double p = pf[b];
                if (clip) p = std::max(0.0, p);
                pp += (p * vol) * W;
                dd += (rho_b * vol) * W;
                ++cnt;
            });
            if (walls)
                foreach_neighbor(gi, wcl, xw.data(), x, sr, [&](int32_t b, const double*, double r) {
                    const double m_b = mw[b];
                    const double vol = m_b / rhow[b];
                    const double W = wc2_kernel(nd, r, hi);
                    if (wall_velocity) shep_w += vol * W;  // wall velocity 0 adds nothing else
                    other += m_b * W;
                    ++cnt;
                });
            const bool cut = rho_c < kEps || (cut_off_bnd && other > rho_c);
            if (cut) {
                cd[i] = NAN;
                count[i] = 0;
                for (int d = 0; d < nd; ++d) vel[i * nd + d] = NAN;
                pres[i] = NAN;
                dens[i] = NAN;
            } else {
                cd[i] = rho_c;
                count[i] = cnt;
                for (int d = 0; d < nd; ++d) vel[i * nd + d] = vv[d] / shep;
                pres[i] = pp / shep;
                dens[i] = dd / shep;
                if (wall_velocity) {
                    const double k = shep_w / shep;
                    for (int d = 0; d < nd; ++d) vel[i * nd + d] /= k;
                }
            }
        }
    }

    // drift! -> set_velocity!, semidiscretization.jl:561-571 (delta_v = 0).
    void drift(T* du, const T* v) const {
        for (int64_t i = 0; i < nf; ++i)
            for (int d = 0; d < nd; ++d) du[i * nd + d] = v[i * (nd + 1) + d];
    }
};

// Carpenter & Kennedy (1994) (5,4) 2N-storage coefficients, solution 3.
const double kA[5] = {0.0,
                      -567301805773.0 / 1357537059087.0,
                      -2404267990393.0 / 2016746695238.0,
                      -3550918686646.0 / 2091501179385.0,
                      -1275806237668.0 / 842570457699.0};
const double kB[5] = {1432997174477.0 / 9575080441755.0,
                      5161836677717.0 / 13612068292357.0,
                      1720146321549.0 / 2090206949498.0,
                      3134564353537.0 / 4481467310338.0,
                      2277821191437.0 / 14882151754819.0};
const double kC[5] = {0.0,
                      1432997174477.0 / 9575080441755.0,
                      2526269341429.0 / 6820363962896.0,
                      2006345519317.0 / 3224310063776.0,
                      2802321613138.0 / 2924317926251.0};

using Model = ModelT<double>;

// n_steps CarpenterKennedy2N54 steps at fixed dt, in place on (v, u); the stage update
// tmp = A_i tmp + dt k; x += B_i tmp with fused multiply-adds (the @muladd of
// OrdinaryDiffEqLowStorageRK).  Returns 0, or 3 if a particle left the grid.
template <class T>
int integrate_ck2n54(ModelT<T>* m, T* v, T* u, double dt, int64_t n_steps) {
    using std::fma;
    const int64_t nvv = m->nf * (m->nd + 1), nuu = m->nf * m->nd;
    std::vector<T> kv(nvv), ku(nuu), tv(nvv), tu(nuu);
    const T dtt = dt;
    int status = 0;
    for (int64_t step = 0; step < n_steps; ++step) {
        for (int s = 0; s < 5; ++s) {
            if (s > 0) {
                for (int64_t i = 0; i < nvv; ++i) tv[i] = kA[s] * tv[i];
                for (int64_t i = 0; i < nuu; ++i) tu[i] = kA[s] * tu[i];
            }
            m->kick(kv.data(), v, u);
            if (!m->grid_ok) status = 3;
            m->drift(ku.data(), v);
            if (s == 0) {
                for (int64_t i = 0; i < nvv; ++i) tv[i] = dt * kv[i];
                for (int64_t i = 0; i < nuu; ++i) tu[i] = dt * ku[i];
            } else {
                for (int64_t i = 0; i < nvv; ++i) tv[i] = fma(dtt, kv[i], tv[i]);
                for (int64_t i = 0; i < nuu; ++i) tu[i] = fma(dtt, ku[i], tu[i]);
            }
            const T bs = kB[s];
            for (int64_t i = 0; i < nvv; ++i) v[i] = fma(bs, tv[i], v[i]);
            for (int64_t i = 0; i < nuu; ++i) u[i] = fma(bs, tu[i], u[i]);
        }
    }
    return status;
}

}  // namespace

// =========================================================================================
// C entry points (ctypes)
// =========================================================================================
extern "C" {

struct orc_model;  // opaque

orc_model* orc_create(const tp_config* cfg, const double* x_wall, const double* m_wall,
                      const double* m_fluid) {
    Model* m = new Model();
    if (!m->init(*cfg)) {
        delete m;
        return nullptr;
    }
    m->xw.assign(x_wall, x_wall + cfg->n_wall * cfg->ndims);
    m->mw.assign(m_wall, m_wall + cfg->n_wall);
    m->mf.assign(m_fluid, m_fluid + cfg->n_fluid);
    m->wall_cl.build(m->grid, m->xw.data(), cfg->n_wall);
    return reinterpret_cast<orc_model*>(m);
}

void orc_destroy(orc_model* p) { delete reinterpret_cast<Model*>(p); }

// One kick! into dv (layout (ndims+1, n_fluid)); returns 0, or 3 if a particle left the grid.
int orc_kick(orc_model* p, double* dv, const double* v, const double* u) {
    Model* m = reinterpret_cast<Model*>(p);
    m->kick(dv, v, u);
    return m->grid_ok ? 0 : 3;
}

void orc_drift(orc_model* p, double* du, const double* v) {
    reinterpret_cast<Model*>(p)->drift(du, v);
}

// Pressures/densities from the last kick (fluid p, wall p, wall rho, wall volume); any may be null.
void orc_last_state(orc_model* p, double* pf, double* pw, double* rhow, double* volw) {
    Model* m = reinterpret_cast<Model*>(p);
    if (pf) std::copy(m->pf.begin(), m->pf.end(), pf);
    if (pw) std::copy(m->pw.begin(), m->pw.end(), pw);
    if (rhow) std::copy(m->rhow.begin(), m->rhow.end(), rhow);
    if (volw) std::copy(m->volw.begin(), m->volw.end(), volw);
}

// n_steps CarpenterKennedy2N54 steps at fixed dt, in place on (v, u).
int orc_integrate_ck2n54(orc_model* p, double* v, double* u, double dt, int64_t n_steps) {
    return integrate_ck2n54(reinterpret_cast<Model*>(p), v, u, dt, n_steps);
}

// Forward-mode derivatives (dual numbers, dual.h) of n_steps CarpenterKennedy2N54 steps from
// (v, u): four directions -- Monaghan alpha, Molteni-Colagrossi delta, the gravity magnitude
// (along the configured acceleration) and the initial state along (v_dir, u_dir) (either may be
// null = zero).  (v, u) are advanced in place (their values equal orc_integrate_ck2n54's);
// dv_out (4 x n_fluid*(ndims+1)) and du_out (4 x n_fluid*ndims) receive the derivatives of
// the final state, direction by direction.  Returns 0, 1 (bad configuration) or 3.
int orc_integrate_ck2n54_jvp(const tp_config* cfg, const double* x_wall, const double* m_wall,
                             const double* m_fluid, double* v, double* u, const double* v_dir,
                             const double* u_dir, double dt, int64_t n_steps, double* dv_out,
                             double* du_out) {
    using D = orc::Dual<4>;
    ModelT<D> m;
    if (!m.init(*cfg)) return 1;
    m.xw.assign(x_wall, x_wall + cfg->n_wall * cfg->ndims);
    m.mw.assign(m_wall, m_wall + cfg->n_wall);
    m.mf.assign(m_fluid, m_fluid + cfg->n_fluid);
    m.wall_cl.build(m.grid, m.xw.data(), cfg->n_wall);
    m.alpha_p.d[0] = 1.0;
    m.delta_p.d[1] = 1.0;
    double gn = 0.0;
    for (int d = 0; d < 3; ++d) gn += cfg->acceleration[d] * cfg->acceleration[d];
    gn = std::sqrt(gn);
    for (int d = 0; d < 3; ++d) m.grav[d].d[2] = gn > 0.0 ? cfg->acceleration[d] / gn : 0.0;
    const int64_t nvv = cfg->n_fluid * (cfg->ndims + 1), nuu = cfg->n_fluid * cfg->ndims;
    std::vector<D> vd(nvv), ud(nuu);
    for (int64_t i = 0; i < nvv; ++i) {
        vd[i] = v[i];
        vd[i].d[3] = v_dir ? v_dir[i] : 0.0;
    }
    for (int64_t i = 0; i < nuu; ++i) {
        ud[i] = u[i];
        ud[i].d[3] = u_dir ? u_dir[i] : 0.0;
    }
    const int st = integrate_ck2n54(&m, vd.data(), ud.data(), dt, n_steps);
    for (int64_t i = 0; i < nvv; ++i) {
        v[i] = vd[i].v;
        for (int k = 0; k < 4; ++k) dv_out[k * nvv + i] = vd[i].d[k];
    }
    for (int64_t i = 0; i < nuu; ++i) {
        u[i] = ud[i].v;
        for (int k = 0; k < 4; ++k) du_out[k * nuu + i] = ud[i].d[k];
    }
    return st;
}

// SymplecticPositionVerlet (ext/TrixiParticlesOrdinaryDiffEqSymplecticRKExt.jl:89-171), the
// @muladd forms as fused multiply-adds:
//   u_h = uprev + (dt/2) v_prev;  v_h = vprev + (dt/2) kick(vprev, uprev);  k = kick(v_h, u_h);
//   v = vprev + dt k (velocity rows);  rho = rho_prev (2 - eps) / (2 + eps),
//   eps = (-k_rho / rho_h) dt;  u = u_h + (dt/2) v.
int orc_integrate_spv(orc_model* p, double* v, double* u, double dt, int64_t n_steps) {
    Model* m = reinterpret_cast<Model*>(p);
    const int nd = m->nd;
    const int64_t nf = m->nf, nvv = nf * (nd + 1), nuu = nf * nd;
    std::vector<double> kv(nvv), ku(nuu), vh(nvv), uh(nuu);
    const double half = 0.5, dth = dt * half;
    int status = 0;
    for (int64_t step = 0; step < n_steps; ++step) {
        m->drift(ku.data(), v);
        for (int64_t i = 0; i < nuu; ++i) uh[i] = std::fma(dth, ku[i], u[i]);
        m->kick(kv.data(), v, u);
        if (!m->grid_ok) status = 3;
        for (int64_t i = 0; i < nvv; ++i) vh[i] = std::fma(dth, kv[i], v[i]);
        m->kick(kv.data(), vh.data(), uh.data());
        if (!m->grid_ok) status = 3;
        for (int64_t a = 0; a < nf; ++a) {
            for (int d = 0; d < nd; ++d)
                v[a * (nd + 1) + d] = std::fma(dt, kv[a * (nd + 1) + d], v[a * (nd + 1) + d]);
            const double rho_prev = v[a * (nd + 1) + nd];
            const double rho_half = vh[a * (nd + 1) + nd];
            const double eps = (-kv[a * (nd + 1) + nd] / rho_half) * dt;
            v[a * (nd + 1) + nd] = rho_prev * (2.0 - eps) / (2.0 + eps);
        }
        m->drift(ku.data(), v);
        for (int64_t i = 0; i < nuu; ++i) u[i] = std::fma(dth, ku[i], uh[i]);
    }
    return status;
}

// SortingCallback's permutation (src/callbacks/sorting.jl:135-158): sortperm over the
// SVector cell coordinates (lexicographic, stable), cells as in the neighbour search.
int orc_sort_perm(const tp_config* cfg, const double* x, int64_t n, int32_t* perm) {
    Grid g;
    if (!g.init(*cfg)) return 1;
    std::vector<std::array<int64_t, 3>> cc(n);
    for (int64_t i = 0; i < n; ++i) {
        int64_t c[3];
        g.cell_of(x + i * g.nd, c);
        cc[i] = {c[0], c[1], c[2]};
    }
    std::vector<int32_t> p(n);
    std::iota(p.begin(), p.end(), 0);
    std::stable_sort(p.begin(), p.end(), [&](int32_t a, int32_t b) { return cc[a] < cc[b]; });
    std::copy(p.begin(), p.end(), perm);
    return 0;
}

void orc_interpolate(orc_model* p, const double* v, const double* u, const double* points,
                     int64_t n_points, double smoothing_length, int cut_off_bnd,
                     int clip_negative_pressure, int include_wall_velocity,
                     double* computed_density, double* velocity, double* pressure,
                     double* density, int32_t* neighbor_count) {
    reinterpret_cast<Model*>(p)->interpolate(v, u, points, n_points, smoothing_length,
                                             cut_off_bnd != 0, clip_negative_pressure != 0,
                                             include_wall_velocity != 0, computed_density,
                                             velocity, pressure, density, neighbor_count);
}

void orc_ck2n54_coefficients(double* A, double* B, double* C) {
    for (int i = 0; i < 5; ++i) {
        A[i] = kA[i];
        B[i] = kB[i];
        C[i] = kC[i];
    }
}

// Neighbour-search diagnostics (same meaning as tp_nhs_debug).
int orc_nhs(const tp_config* cfg, const double* x_fluid, const double* x_wall, int32_t* cell,
            int32_t* order, int32_t* nnb_ff, int32_t* nnb_fw, int32_t* nnb_wf) {
    Grid g;
    if (!g.init(*cfg)) return 1;
    CellList fl, wl;
    const int64_t nf = cfg->n_fluid, nw = cfg->n_wall;
    const int nd = cfg->ndims;
    fl.build(g, x_fluid, nf);
    wl.build(g, x_wall, nw);
    const double sr = 2.0 * cfg->smoothing_length;
    if (cell) std::copy(fl.key.begin(), fl.key.end(), cell);
    if (order) std::copy(fl.order.begin(), fl.order.end(), order);
#pragma omp parallel for schedule(static)
    for (int64_t a = 0; a < nf; ++a) {
        int32_t cf = 0, cw = 0;
        foreach_neighbor(g, fl, x_fluid, x_fluid + a * nd, sr,
                         [&](int32_t, const double*, double) { ++cf; });
        foreach_neighbor(g, wl, x_wall, x_fluid + a * nd, sr,
                         [&](int32_t, const double*, double) { ++cw; });
        if (nnb_ff) nnb_ff[a] = cf;
        if (nnb_fw) nnb_fw[a] = cw;
    }
#pragma omp parallel for schedule(static)
    for (int64_t w = 0; w < nw; ++w) {
        int32_t c = 0;
        foreach_neighbor(g, fl, x_fluid, x_wall + w * nd, sr,
                         [&](int32_t, const double*, double) { ++c; });
        if (nnb_wf) nnb_wf[w] = c;
    }
    return (fl.ok && wl.ok) ? 0 : 3;
}

// ---- Known-answer helpers ----
double orc_wendland_c2(int nd, double r, double h) { return wc2_kernel(nd, r, h); }
double orc_wendland_c2_deriv_div_r(int nd, double r, double h) {
    return wc2_deriv_div_r(nd, r, h);
}
double orc_cole_pressure(double c, double rho0, double gamma, double p_bg, int clip, double rho) {
    Eos e{rho0, c, gamma, p_bg, clip != 0};
    return e.pressure(rho);
}
double orc_cole_inverse(double c, double rho0, double gamma, double p_bg, double p) {
    Eos e{rho0, c, gamma, p_bg, false};
    return e.inverse(p);
}

// ArtificialViscosityMonaghan single pair (viscosity.jl:99-132) with SchoenbergCubicSpline{nd}
// gradient; reproduces test/schemes/fluid/viscosity.jl:18-42.
void orc_monaghan_pair(int nd, double h, double c, double alpha, double beta, double eps,
                       const double* pos_diff, const double* v_a, const double* v_b,
                       double m_b, double rho_a, double rho_b, double* dv_out) {
    double d2 = dot(nd, pos_diff, pos_diff);
    double r = std::sqrt(d2);
    // smoothing_kernel_grad (abstract_system.jl:140-153): checks then unsafe gradient.
    double grad[3] = {0, 0, 0};
    if (!(r >= 2.0 * h || d2 < (std::nextafter(h * h, INFINITY) - h * h))) {
        double s = scs_deriv_div_r(nd, r, h);
        for (int d = 0; d < nd; ++d) grad[d] = s * pos_diff[d];
    }
    double vd[3] = {v_a[0] - v_b[0], v_a[1] - v_b[1], nd == 3 ? v_a[2] - v_b[2] : 0.0};
    double vr = dot(nd, vd, pos_diff);
    for (int d = 0; d < nd; ++d) dv_out[d] = 0.0;
    if (vr < 0.0) {
        double hh = (h + h) / 2.0;
        double rho_mean = (rho_a + rho_b) / 2.0;
        double mu = (hh * vr) / (r * r + eps * (hh * hh));
        double num = ((m_b * alpha) * c) * mu + (m_b * beta) * (mu * mu);
        double f = num / rho_mean;
        for (int d = 0; d < nd; ++d) dv_out[d] = 0.0 + f * grad[d];
    }
}

// ---- RectangularTank restatement (src/setups/rectangular_tank.jl, rectangular_shape.jl) ----
// Julia's round(Int, x): ties to even.
static int64_t jl_round(double x) { return (int64_t)std::nearbyint(x); }

static bool jl_isapprox(double a, double b) {
    double rtol = std::sqrt(kEps);
    return std::fabs(a - b) <= rtol * std::max(std::fabs(a), std::fabs(b));
}

// rectangular_shape_coords (rectangular_shape.jl:196-224) with loop_permutation (:168-194);
// loop: 0 = default/(y_first in 2D, z_first in 3D), 'x' / 'y' / 'z' as in the reference.
static void shape_coords(int nd, double dx, const int64_t* np, const double* mc, char loop,
                         std::vector<double>& out) {
    // permutation p: linear iteration over permutedims(CartesianIndices(np), p); the first
    // dimension of the permuted array (index p[0]) runs fastest.
    int p[3] = {0, 1, 2};
    if (nd == 2) {
        if (loop == 'x') { p[0] = 1; p[1] = 0; }
    } else {
        if (loop == 'y') { p[0] = 1; p[1] = 0; p[2] = 2; }
        else if (loop == 'x') { p[0] = 2; p[1] = 1; p[2] = 0; }
    }
    int64_t np3[3] = {np[0], np[1], nd == 3 ? np[2] : 1};
    int64_t idx[3];
    int64_t n0 = np3[p[0]], n1 = np3[p[1]], n2 = (nd == 3) ? np3[p[2]] : 1;
    for (int64_t k2 = 0; k2 < n2; ++k2)
        for (int64_t k1 = 0; k1 < n1; ++k1)
            for (int64_t k0 = 0; k0 < n0; ++k0) {
                idx[p[0]] = k0;
                idx[p[1]] = k1;
                if (nd == 3) idx[p[2]] = k2;
                for (int d = 0; d < nd; ++d)
                    out.push_back(mc[d] + dx * ((double)(idx[d] + 1) - 0.5));
            }
}

// Counts of a closed tank (all faces).  Returns n_fluid, n_wall.
// faces: 2*nd booleans (-x,+x,-y,+y[,-z,+z]).
int orc_tank(int nd, double dx, const double* fluid_size, const double* tank_size, int n_layers,
             const int32_t* faces, double rho0, double c, double gamma, double p_bg,
             const double* accel, int64_t* n_fluid, int64_t* n_wall, double* x_f,
             double* rho_f, double* m_f, double* x_w, double* rho_w, double* m_w) {
    int64_t nfd[3] = {1, 1, 1}, nbd[3] = {1, 1, 1};
    double fsz[3] = {0, 0, 0}, tsz[3] = {0, 0, 0};
    for (int d = 0; d < nd; ++d) {
        nfd[d] = jl_round(fluid_size[d] / dx);
        fsz[d] = (double)nfd[d] * dx;
        tsz[d] = tank_size[d];
    }
    for (int d = 0; d < nd; ++d)
        if (jl_isapprox(fluid_size[d], tank_size[d])) tsz[d] = fsz[d];
    const double bdx = dx / 1.0;  // spacing_ratio = 1
    for (int d = 0; d < nd; ++d) {
        nbd[d] = jl_round(tsz[d] / bdx);
        tsz[d] = (double)nbd[d] * bdx;
    }
    // check_tank_overlap (rectangular_tank.jl:474-528)
    for (int d = 0; d < nd; ++d)
        if (tsz[d] < fsz[d] - 1e-5 * dx) {
            nfd[d] -= 1;
            fsz[d] = (double)nfd[d] * dx;
        }
    // initialize_boundaries (rectangular_tank.jl:530-690 and 3D equivalent)
    std::vector<double> wc;
    const double lo = -(double)n_layers * bdx;
    const int64_t L = n_layers;
    auto F = [&](int i) { return faces[i] != 0; };
    if (nd == 2) {
        int64_t nx = nbd[0], ny = nbd[1];
        if (F(0)) { int64_t n[2] = {L, ny}; double m[2] = {lo, 0.0}; shape_coords(2, bdx, n, m, 'x', wc); }
        if (F(1)) { int64_t n[2] = {L, ny}; double m[2] = {tsz[0], 0.0}; shape_coords(2, bdx, n, m, 'x', wc); }
        if (F(2)) { int64_t n[2] = {nx, L}; double m[2] = {0.0, lo}; shape_coords(2, bdx, n, m, 'y', wc); }
        if (F(3)) { int64_t n[2] = {nx, L}; double m[2] = {0.0, tsz[1]}; shape_coords(2, bdx, n, m, 'y', wc); }
        int64_t nc[2] = {L, L};
        if (F(0) && F(2)) { double m[2] = {lo, lo}; shape_coords(2, bdx, nc, m, 0, wc); }
        if (F(0) && F(3)) { double m[2] = {lo, tsz[1]}; shape_coords(2, bdx, nc, m, 0, wc); }
        if (F(1) && F(2)) { double m[2] = {tsz[0], lo}; shape_coords(2, bdx, nc, m, 0, wc); }
        if (F(1) && F(3)) { double m[2] = {tsz[0], tsz[1]}; shape_coords(2, bdx, nc, m, 0, wc); }
    } else {
        int64_t nx = nbd[0], ny = nbd[1], nz = nbd[2];
        const int left = 0, right = 1, bottom = 2, top = 3, front = 4, back = 5;
        auto S = [&](int64_t a, int64_t b, int64_t c3, double m0, double m1, double m2, char lp) {
            int64_t n[3] = {a, b, c3};
            double m[3] = {m0, m1, m2};
            shape_coords(3, bdx, n, m, lp, wc);
        };
        // faces
        if (F(left)) S(L, ny, nz, lo, 0.0, 0.0, 'x');
        if (F(right)) S(L, ny, nz, tsz[0], 0.0, 0.0, 'x');
        if (F(bottom)) S(nx, L, nz, 0.0, lo, 0.0, 'y');
        if (F(top)) S(nx, L, nz, 0.0, tsz[1], 0.0, 'y');
        if (F(front)) S(nx, ny, L, 0.0, 0.0, lo, 'z');
        if (F(back)) S(nx, ny, L, 0.0, 0.0, tsz[2], 'z');
        // edges: z-aligned, x-aligned, y-aligned (default loop order)
        if (F(left) && F(bottom)) S(L, L, nz, lo, lo, 0.0, 0);
        if (F(left) && F(top)) S(L, L, nz, lo, tsz[1], 0.0, 0);
        if (F(right) && F(bottom)) S(L, L, nz, tsz[0], lo, 0.0, 0);
        if (F(right) && F(top)) S(L, L, nz, tsz[0], tsz[1], 0.0, 0);
        if (F(front) && F(bottom)) S(nx, L, L, 0.0, lo, lo, 0);
        if (F(front) && F(top)) S(nx, L, L, 0.0, tsz[1], lo, 0);
        if (F(back) && F(bottom)) S(nx, L, L, 0.0, lo, tsz[2], 0);
        if (F(back) && F(top)) S(nx, L, L, 0.0, tsz[1], tsz[2], 0);
        if (F(left) && F(front)) S(L, ny, L, lo, 0.0, lo, 0);
        if (F(left) && F(back)) S(L, ny, L, lo, 0.0, tsz[2], 0);
        if (F(right) && F(front)) S(L, ny, L, tsz[0], 0.0, lo, 0);
        if (F(right) && F(back)) S(L, ny, L, tsz[0], 0.0, tsz[2], 0);
        // corners
        if (F(left) && F(bottom) && F(front)) S(L, L, L, lo, lo, lo, 0);
        if (F(left) && F(top) && F(front)) S(L, L, L, lo, tsz[1], lo, 0);
        if (F(left) && F(bottom) && F(back)) S(L, L, L, lo, lo, tsz[2], 0);
        if (F(left) && F(top) && F(back)) S(L, L, L, lo, tsz[1], tsz[2], 0);
        if (F(right) && F(bottom) && F(front)) S(L, L, L, tsz[0], lo, lo, 0);
        if (F(right) && F(top) && F(front)) S(L, L, L, tsz[0], tsz[1], lo, 0);
        if (F(right) && F(bottom) && F(back)) S(L, L, L, tsz[0], lo, tsz[2], 0);
        if (F(right) && F(top) && F(back)) S(L, L, L, tsz[0], tsz[1], tsz[2], 0);
    }
    int64_t nw = (int64_t)wc.size() / nd;
    int64_t nf = nfd[0] * nfd[1] * (nd == 3 ? nfd[2] : 1);
    *n_fluid = nf;
    *n_wall = nw;
    if (!x_f) return 0;  // count-only call
    // boundary masses / densities (rectangular_tank.jl:150-152): rho0 * dx^d * 1
    double bvol = (nd == 2) ? bdx * bdx : (bdx * bdx) * bdx;
    double bmass = rho0 * bvol;
    std::copy(wc.begin(), wc.end(), x_w);
    for (int64_t i = 0; i < nw; ++i) {
        rho_w[i] = rho0 * 1.0;
        m_w[i] = bmass * 1.0;
    }
    // fluid (RectangularShape with hydrostatic pressure, rectangular_shape.jl:79-154, 226-267)
    std::vector<double> fc;
    double zero[3] = {0.0, 0.0, 0.0};
    shape_coords(nd, dx, nfd, zero, 0, fc);
    std::copy(fc.begin(), fc.end(), x_f);
    Eos eos{rho0, c, gamma, p_bg, false};
    int ad = -1;
    for (int d = 0; d < nd; ++d)
        if (std::fabs(accel[d]) > kEps) { ad = d; break; }
    std::vector<double> p1d;
    if (ad >= 0) {
        double factor = dx * std::fabs(accel[ad]);
        p1d.assign(nfd[ad], 0.0);
        p1d[0] = (0.5 * factor) * eos.inverse(0.0);
        for (int64_t i = 0; i + 1 < nfd[ad]; ++i) p1d[i + 1] = p1d[i] + factor * eos.inverse(p1d[i]);
        if (accel[ad] < 0) std::reverse(p1d.begin(), p1d.end());
    }
    double fvol = (nd == 2) ? dx * dx : (dx * dx) * dx;
    for (int64_t i = 0; i < nf; ++i) {
        double p = 0.0;
        if (ad >= 0) {
            // default loop order: x fastest, then y, then z
            int64_t k = i;
            int64_t id[3];
            id[0] = k % nfd[0];
            k /= nfd[0];
            id[1] = k % nfd[1];
            k /= nfd[1];
            id[2] = k;
            p = p1d[id[ad]];
        }
        rho_f[i] = eos.inverse(p);
        m_f[i] = fvol * rho_f[i];
    }
    return 0;
}

}  // extern "C"
