// tp_interp.cu — SPH interpolation at arbitrary points (interpolate_points / interpolate_line,
// src/general/interpolation.jl:381-697) on sm_103a.
//
// One thread per point gathers the fluid particles (and, with cut_off_bnd or
// include_wall_velocity, the wall particles) within the interpolation support 2 h_i from the
// handle's cell grid (cell size 2h, so the support spans ceil(h_i / h) cells each side):
//   computed_density = sum m_b W,   shepard = sum V_b W (V_b = m_b / rho_b),
//   velocity / pressure / density = sum f_b V_b W / shepard   (pressure clipped at 0 on request),
//   other_density = sum over walls m_w W,   neighbor_count = particles within the support;
// points with computed_density < eps() (or, with cut_off_bnd, other_density > computed_density)
// get NaN fields and a zero count.  With include_wall_velocity the velocity is renormalised by
// shepard / (shepard + sum_walls V_w W) (wall velocity is zero here: fixed walls).
// FP64 throughout in both precision forms; the fluid state is read in caller order, the fluid
// pressure is the Cole EOS of the current density, the wall density that of the Adami pass run
// on the same state just before.  Sums run in cell-grid order, so they equal the reference's to
// rounding (the reference visits cells of size 2 h_i).
#include "tp_api_internal.h"
#include "tp_lists.cuh"

namespace tp {

struct InterpArgs {
    GridDesc g;
    Phys P;
    int reach;
    double hi, sr2, norm, h_inv;
    long long np;
    const double* pts;
    const double* u;
    const double* v;
    const double* mf;
    const int* fperm;
    const int* fstart;
    int nw;
    const double4_32a* wpos;
    const int* wstart;
    const void* wstate;
    int f32;
    int walls, cut_off_bnd, clip, wall_velocity;
    double* cd;
    double* vel;
    double* pres;
    double* dens;
    int* count;
};

__device__ __forceinline__ double wc2_w(double r, const InterpArgs& A) {
    if (!(r < 2.0 / A.h_inv)) return 0.0;
    const double q = r * A.h_inv;
    const double t = 1.0 - q / 2.0;
    const double t2 = t * t;
    return (A.norm * (t2 * t2)) * (2.0 * q + 1.0);
}

template <int ND>
__global__ void __launch_bounds__(128) k_interpolate(InterpArgs A) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.np) return;
    double x[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int d = 0; d < ND; ++d) x[d] = A.pts[i * ND + d];
    int c[3];
    cell_coords<ND>(x, A.g, c);  // clamped into the grid; points must lie inside its box
    double rho_c = 0.0, other = 0.0, shep = 0.0, shep_w = 0.0, pp = 0.0, dd = 0.0;
    double vv[3] = {0.0, 0.0, 0.0};
    int cnt = 0;
    const int zr = (ND == 3) ? A.reach : 0;
    const int xlo = max(c[0] - A.reach, 0), xhi = min(c[0] + A.reach, A.g.n[0] - 1);
    for (int dz = -zr; dz <= zr; ++dz) {
        const int cz = c[2] + dz;
        if (cz < 0 || cz >= A.g.n[2]) continue;
        for (int dy = -A.reach; dy <= A.reach; ++dy) {
            const int cy = c[1] + dy;
            if (cy < 0 || cy >= A.g.n[1]) continue;
            const int row = A.g.n[0] * (cy + A.g.n[1] * cz);
            for (int s = A.fstart[row + xlo]; s < A.fstart[row + xhi + 1]; ++s) {
                const int b = A.fperm[s];
                double d2 = 0.0;
#pragma unroll
                for (int d = 0; d < ND; ++d) {
                    const double e = x[d] - A.u[(size_t)b * ND + d];
                    d2 += e * e;
                }
                if (d2 > A.sr2) continue;
                const double W = wc2_w(sqrt(d2), A);
                const double m = A.mf[b];
                const double rho = A.v[(size_t)b * (ND + 1) + ND];
                const double vol = m / rho;
                if (A.wall_velocity) shep_w += vol * W;
                rho_c += m * W;
                shep += vol * W;
#pragma unroll
                for (int d = 0; d < ND; ++d) vv[d] += (A.v[(size_t)b * (ND + 1) + d] * vol) * W;
                double p = eos_pressure(rho, A.P, A.P.fluid_clip);
                if (A.clip) p = fmax(0.0, p);
                pp += (p * vol) * W;
                dd += (rho * vol) * W;
                ++cnt;
            }
            if (!A.walls) continue;
            for (int w = A.wstart[row + xlo]; w < A.wstart[row + xhi + 1]; ++w) {
                const double4_32a pw = A.wpos[w];
                const double xw[3] = {pw.x, pw.y, pw.z};
                double d2 = 0.0;
#pragma unroll
                for (int d = 0; d < ND; ++d) {
                    const double e = x[d] - xw[d];
                    d2 += e * e;
                }
                if (d2 > A.sr2) continue;
                const double W = wc2_w(sqrt(d2), A);
                if (A.wall_velocity) {
                    const double rho_w = A.f32 ? (double)((const float4*)A.wstate)[w].y + A.P.rho0
                                               : ((const double4_32a*)A.wstate)[w].y;
                    shep_w += (pw.w / rho_w) * W;
                }
                other += pw.w * W;
                ++cnt;
            }
        }
    }
    const bool cut = rho_c < 2.220446049250313e-16 || (A.cut_off_bnd && other > rho_c);
    if (cut) {
        const double nan = __longlong_as_double(0x7ff8000000000000LL);  // quiet NaN
        A.cd[i] = nan;
        A.count[i] = 0;
#pragma unroll
        for (int d = 0; d < ND; ++d) A.vel[i * ND + d] = nan;
        A.pres[i] = nan;
        A.dens[i] = nan;
        return;
    }
    A.cd[i] = rho_c;
    A.count[i] = cnt;
    const double k = A.wall_velocity ? shep_w / shep : 1.0;
#pragma unroll
    for (int d = 0; d < ND; ++d) {
        double val = vv[d] / shep;
        if (A.wall_velocity) val /= k;
        A.vel[i * ND + d] = val;
    }
    A.pres[i] = pp / shep;
    A.dens[i] = dd / shep;
}

void interp_launch(tp_handle* h, const double* v, const double* u, const double* pts,
                   long long np, double hi, int walls, int cut_off_bnd, int clip,
                   int wall_velocity, double* cd, double* vel, double* pres, double* dens,
                   int* count) {
    InterpArgs A{};
    A.g = h->grid;
    A.P = h->phys;
    A.hi = hi;
    A.h_inv = 1.0 / hi;
    A.norm = (h->cfg.ndims == 2) ? (7.0 / (4.0 * 3.141592653589793)) * (A.h_inv * A.h_inv)
                                 : (21.0 / (16.0 * 3.141592653589793)) *
                                       ((A.h_inv * A.h_inv) * A.h_inv);
    A.sr2 = (2.0 * hi) * (2.0 * hi);
    A.reach = (int)std::ceil(2.0 * hi / h->grid.cs - 1e-12);
    if (A.reach < 1) A.reach = 1;
    A.np = np;
    A.pts = pts;
    A.u = u;
    A.v = v;
    A.mf = h->m_f;
    A.fperm = h->f_perm;
    A.fstart = h->f_start;
    A.nw = (int)h->cfg.n_wall;
    A.wpos = (const double4_32a*)h->w_pos;
    A.wstart = h->w_start;
    A.wstate = h->w_state;
    A.f32 = h->cfg.precision == TP_PRECISION_FP32;
    A.walls = walls && A.nw > 0;
    A.cut_off_bnd = cut_off_bnd;
    A.clip = clip;
    A.wall_velocity = wall_velocity;
    A.cd = cd;
    A.vel = vel;
    A.pres = pres;
    A.dens = dens;
    A.count = count;
    const int blocks = (int)((np + 127) / 128);
    if (h->cfg.ndims == 2)
        k_interpolate<2><<<blocks, 128, 0, h->stream>>>(A);
    else
        k_interpolate<3><<<blocks, 128, 0, h->stream>>>(A);
    h->launches += 1;
}

}  // namespace tp
