// tp_api.cu — C ABI of the sm_103a WCSPH library: handle, neighbour-search orchestration,
// kick!/drift! and the fused CarpenterKennedy2N54 integrator.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "tp_api_internal.h"
#include "tp_lists.cuh"

using namespace tp;

namespace {

std::string g_create_error;  // message of the last failed tp_create

inline int nblk(long n, int t) { return (int)((n + t - 1) / t); }

tp_status fail(tp_handle* h, tp_status st, const std::string& msg) {
    if (h) h->last_error = msg;
    return st;
}

tp_status cuda_fail(tp_handle* h, cudaError_t e, const char* where) {
    std::string m = std::string(where) + ": " + cudaGetErrorString(e);
    return fail(h, TP_ERR_CUDA, m);
}

#define TP_CUDA(h, call)                                   \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return cuda_fail(h, e_, #call); \
    } while (0)

#define TP_LAUNCHED(h, where)                              \
    do {                                                   \
        cudaError_t e_ = cudaGetLastError();               \
        if (e_ != cudaSuccess) return cuda_fail(h, e_, where); \
    } while (0)

// TP_DEBUG_SYNC=1: synchronise and check after every launch group and print a progress line to
// stderr (diagnostics of a failing launch; never set in production runs).
bool debug_sync_enabled() {
    static const bool on = [] {
        const char* e = std::getenv("TP_DEBUG_SYNC");
        return e && e[0] == '1';
    }();
    return on;
}

tp_status dbg(tp_handle* h, const char* what) {
    if (!debug_sync_enabled()) return TP_OK;
    std::fprintf(stderr, "tp: %s ...", what);
    std::fflush(stderr);
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e == cudaSuccess) e = cudaGetLastError();
    std::fprintf(stderr, " %s\n", e == cudaSuccess ? "ok" : cudaGetErrorString(e));
    std::fflush(stderr);
    if (e != cudaSuccess) return cuda_fail(h, e, what);
    return TP_OK;
}

#define TP_DBG(h, what)                      \
    do {                                     \
        tp_status s_ = dbg((h), (what));     \
        if (s_ != TP_OK) return s_;          \
    } while (0)

template <class T>
cudaError_t dalloc(T** p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    return cudaMalloc((void**)p, n * sizeof(T));
}

// CarpenterKennedy2N54 (Carpenter & Kennedy 1994, (5,4) 2N-storage, solution 3).
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

// ---------------------------------------------------------------------------------------
// Small kernels of the API layer
// ---------------------------------------------------------------------------------------
template <int ND>
__global__ void k_drift(double* __restrict__ du, const double* __restrict__ v, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
#pragma unroll
    for (int d = 0; d < ND; ++d) du[(size_t)i * ND + d] = v[(size_t)i * (ND + 1) + d];
}

// Gather of the caller-ordered state into the order perm (new j <- old perm[j]).
template <int ND>
__global__ void k_permute_state(const int* __restrict__ perm, const double* __restrict__ v,
                                const double* __restrict__ u, const double* __restrict__ m,
                                double* __restrict__ v2, double* __restrict__ u2,
                                double* __restrict__ m2, int n) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int i = perm[j];
#pragma unroll
    for (int d = 0; d <= ND; ++d) v2[(size_t)j * (ND + 1) + d] = v[(size_t)i * (ND + 1) + d];
#pragma unroll
    for (int d = 0; d < ND; ++d) u2[(size_t)j * ND + d] = u[(size_t)i * ND + d];
    if (m2) m2[j] = m[i];
}

// SymplecticPositionVerlet pieces (the @muladd forms as fma):
// u_h = u + (dt/2) v[0:nd]
template <int ND>
__global__ void k_spv_half_drift(const double* __restrict__ u, const double* __restrict__ v,
                                 double dth, double* __restrict__ uh, int n) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
#pragma unroll
    for (int d = 0; d < ND; ++d)
        uh[(size_t)a * ND + d] = fma(dth, v[(size_t)a * (ND + 1) + d], u[(size_t)a * ND + d]);
}

// v_h = v + (dt/2) k (all rows)
__global__ void k_spv_half_kick(const double* __restrict__ v, const double* __restrict__ k,
                                double dth, double* __restrict__ vh, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) vh[i] = fma(dth, k[i], v[i]);
}

// v = v + dt k (velocity rows); rho = rho (2 - eps) / (2 + eps), eps = (-k_rho / rho_h) dt;
// u = u_h + (dt/2) v
template <int ND>
__global__ void k_spv_finish(double* __restrict__ v, double* __restrict__ u,
                             const double* __restrict__ k, const double* __restrict__ vh,
                             const double* __restrict__ uh, double dt, double dth, int n) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    double* va = v + (size_t)a * (ND + 1);
    const double* ka = k + (size_t)a * (ND + 1);
#pragma unroll
    for (int d = 0; d < ND; ++d) va[d] = fma(dt, ka[d], va[d]);
    const double eps = (-ka[ND] / vh[(size_t)a * (ND + 1) + ND]) * dt;
    va[ND] = va[ND] * (2.0 - eps) / (2.0 + eps);
#pragma unroll
    for (int d = 0; d < ND; ++d) u[(size_t)a * ND + d] = fma(dth, va[d], uh[(size_t)a * ND + d]);
}

// Warm start of the integrator: slot s takes caller particle id[s] (the previous call's slot
// order), so the lists of that call stay valid.
template <int ND, bool F32>
__global__ void k_gather_load(const int* __restrict__ id, const double* __restrict__ u,
                              const double* __restrict__ v, const double* __restrict__ m,
                              double rho0, double* __restrict__ su, void* __restrict__ sv,
                              void* __restrict__ sm, int n) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int i = id[s];
#pragma unroll
    for (int d = 0; d < ND; ++d) su[(size_t)s * ND + d] = u[(size_t)i * ND + d];
    const double* vv = v + (size_t)i * (ND + 1);
    if (F32) {
        ((float4*)sv)[s] = make_float4((float)vv[0], (float)vv[1], ND == 3 ? (float)vv[2] : 0.0f,
                                       (float)(vv[ND] - rho0));
        ((float*)sm)[s] = (float)m[i];
    } else {
#pragma unroll
        for (int d = 0; d <= ND; ++d) ((double*)sv)[(size_t)s * (ND + 1) + d] = vv[d];
        ((double*)sm)[s] = m[i];
    }
}

// Rebuild gate {forced, largest squared displacement, squared threshold, largest squared
// displacement of the next stage} for a displacement threshold (skin * h); k_displacement fills
// gate[1], the integrator's pair stage gate[3].
__global__ void k_gate_init(unsigned* __restrict__ gate, float threshold, int force) {
    if (threadIdx.x == 0) {
        gate[0] = force ? 1u : 0u;
        gate[1] = 0u;
        gate[2] = __float_as_uint((threshold * threshold) * (1.0f - 1e-5f));
        gate[3] = 0u;
    }
}

// Integrator, between stages: the forced flag is consumed, the displacement the last pair stage
// collected becomes this stage's, and the next stage's word starts from zero.
__global__ void k_gate_advance(unsigned* __restrict__ gate) {
    if (threadIdx.x == 0) {
        gate[0] = 0u;
        gate[1] = gate[3];
        gate[3] = 0u;
    }
}

__global__ void k_iota(int* __restrict__ id, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) id[i] = i;
}

// FP32 form: caller FP64 (v, rho) and masses -> float4 {v, rho - rho0}, float m.
template <int ND>
__global__ void k_load32(const double* __restrict__ v, const double* __restrict__ m, double rho0,
                         float4* __restrict__ v32, float* __restrict__ m32, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* vv = v + (size_t)i * (ND + 1);
    v32[i] = make_float4((float)vv[0], (float)vv[1], ND == 3 ? (float)vv[2] : 0.0f,
                         (float)(vv[ND] - rho0));
    m32[i] = (float)m[i];
}

// Slot-ordered integrator state -> caller order.
template <int ND, bool F32>
__global__ void k_store(const double* __restrict__ u, const void* __restrict__ v,
                        const int* __restrict__ id, double rho0, double* __restrict__ u_out,
                        double* __restrict__ v_out, int n) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int i = id[s];
#pragma unroll
    for (int d = 0; d < ND; ++d) u_out[(size_t)i * ND + d] = u[(size_t)s * ND + d];
    if (F32) {
        const float4 w = ((const float4*)v)[s];
        const float a[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int d = 0; d < ND; ++d) v_out[(size_t)i * (ND + 1) + d] = (double)a[d];
        v_out[(size_t)i * (ND + 1) + ND] = rho0 + (double)w.w;
    } else {
        const double* vv = (const double*)v;
#pragma unroll
        for (int d = 0; d <= ND; ++d)
            v_out[(size_t)i * (ND + 1) + d] = vv[(size_t)s * (ND + 1) + d];
    }
}

__global__ void k_scatter_pressure(const double4_32a* __restrict__ rec, const int* __restrict__ perm,
                                   double* __restrict__ p, int n) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    p[perm[s]] = rec[s].w;
}

template <bool F32>
__global__ void k_scatter_wall(const void* __restrict__ state, const double* __restrict__ vol,
                               const int* __restrict__ perm, double rho0, double* __restrict__ p,
                               double* __restrict__ rho, double* __restrict__ volume, int n) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int i = perm[s];
    double ps, rs;
    if (F32) {
        const float4 st = ((const float4*)state)[s];
        ps = st.x;
        rs = rho0 + (double)st.y;
    } else {
        const double4_32a st = ((const double4_32a*)state)[s];
        ps = st.x;
        rs = st.y;
    }
    if (p) p[i] = ps;
    if (rho) rho[i] = rs;
    if (volume) volume[i] = vol[s];
}

// FP64 conservation partial sums per block: mass, momentum (3), kinetic energy.
template <int ND>
__global__ void __launch_bounds__(256) k_conservation(const double* __restrict__ v,
                                                      const double* __restrict__ m, int n,
                                                      double* __restrict__ partial) {
    __shared__ double sm[5][8];
    double acc[5] = {0, 0, 0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double mi = m[i];
        double e = 0.0;
        acc[0] += mi;
#pragma unroll
        for (int d = 0; d < ND; ++d) {
            const double vd = v[(size_t)i * (ND + 1) + d];
            acc[1 + d] += mi * vd;
            e += vd * vd;
        }
        acc[4] += 0.5 * mi * e;
    }
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        double x = acc[k];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
        if ((threadIdx.x & 31) == 0) sm[k][threadIdx.x >> 5] = x;
    }
    __syncthreads();
    if (threadIdx.x < 5) {
        double x = 0.0;
        for (int w = 0; w < 8; ++w) x += sm[threadIdx.x][w];
        partial[blockIdx.x * 5 + threadIdx.x] = x;
    }
}

// ---------------------------------------------------------------------------------------
// Host helpers
// ---------------------------------------------------------------------------------------
tp_status check_config(const tp_config* c, std::string& msg) {
    if (!c) { msg = "null config"; return TP_ERR_ARGUMENT; }
    if (c->ndims != 2 && c->ndims != 3) { msg = "ndims must be 2 or 3"; return TP_ERR_ARGUMENT; }
    if (c->precision != TP_PRECISION_FP64 && c->precision != TP_PRECISION_FP32) {
        msg = "precision must be TP_PRECISION_FP64 or TP_PRECISION_FP32";
        return TP_ERR_ARGUMENT;
    }
    if (c->n_fluid < 0 || c->n_wall < 0 || c->n_fluid >= (int64_t(1) << kSlotBits) ||
        c->n_wall >= (int64_t(1) << kSlotBits)) {
        msg = "particle counts must be in [0, 2^25)";
        return TP_ERR_ARGUMENT;
    }
    if (!(c->smoothing_length > 0.0) || !std::isfinite(c->smoothing_length)) {
        msg = "smoothing_length must be positive and finite";
        return TP_ERR_ARGUMENT;
    }
    if (!(c->reference_density > 0.0) || !(c->sound_speed > 0.0) || !(c->exponent > 0.0)) {
        msg = "reference_density, sound_speed and exponent must be positive";
        return TP_ERR_ARGUMENT;
    }
    if (c->viscosity_model != TP_VISCOSITY_NONE && c->viscosity_model != TP_VISCOSITY_MONAGHAN) {
        msg = "unsupported viscosity model";
        return TP_ERR_UNSUPPORTED;
    }
    if (c->density_diffusion_model != TP_DIFFUSION_NONE &&
        c->density_diffusion_model != TP_DIFFUSION_MOLTENI_COLAGROSSI) {
        msg = "unsupported density diffusion model";
        return TP_ERR_UNSUPPORTED;
    }
    for (int d = 0; d < c->ndims; ++d) {
        if (!std::isfinite(c->min_corner[d]) || !std::isfinite(c->max_corner[d]) ||
            !(c->min_corner[d] <= c->max_corner[d])) {
            msg = "FullGridCellList bounds must be finite with min_corner <= max_corner";
            return TP_ERR_ARGUMENT;
        }
    }
    return TP_OK;
}

void setup_phys(tp_handle* h) {
    const tp_config& c = h->cfg;
    Phys& P = h->phys;
    const double pi = 3.141592653589793;
    P.nd = c.ndims;
    P.h = c.smoothing_length;
    P.h_inv = 1.0 / P.h;
    P.two_h = 2.0 * P.h;
    P.sr2 = P.two_h * P.two_h;
    P.almostzero = std::sqrt(std::nextafter(P.sr2, INFINITY) - P.sr2);
    P.az2 = std::nextafter(P.sr2, INFINITY) - P.sr2;
    P.hi2 = P.h_inv * P.h_inv;
    P.wc2_norm = (c.ndims == 2) ? (7.0 / (4.0 * pi)) * (P.h_inv * P.h_inv)
                                : (21.0 / (16.0 * pi)) * ((P.h_inv * P.h_inv) * P.h_inv);
    P.wc2_dnorm = -5.0 * P.wc2_norm;
    P.rho0 = c.reference_density;
    P.c = c.sound_speed;
    P.gamma = c.exponent;
    P.gamma_int = (c.exponent >= 1.0 && c.exponent <= 16.0 && c.exponent == std::floor(c.exponent))
                      ? (int)c.exponent : 0;
    P.p_bg = c.background_pressure;
    P.B = (P.rho0 * (P.c * P.c)) / P.gamma;
    P.inv_gamma = 1.0 / P.gamma;
    P.fluid_clip = c.fluid_clip_negative_pressure != 0;
    P.wall_clip = c.wall_clip_negative_pressure != 0;
    P.visc = c.viscosity_model == TP_VISCOSITY_MONAGHAN;
    P.alpha = c.viscosity_alpha;
    P.beta = c.viscosity_beta;
    P.eps_visc = c.viscosity_epsilon;
    P.visc_h = (P.h + P.h) / 2.0;
    P.visc_eps_h2 = P.eps_visc * (P.visc_h * P.visc_h);
    P.visc_mac = P.alpha * P.c;
    P.diff = c.density_diffusion_model == TP_DIFFUSION_MOLTENI_COLAGROSSI;
    P.delta = c.density_diffusion_delta;
    P.diff_coef = (P.delta * ((P.h + P.h) / 2.0)) * P.c;
    for (int d = 0; d < 3; ++d) P.g[d] = (d < c.ndims) ? c.acceleration[d] : 0.0;
    P.p_off = c.pressure_offset;
    P.sg_c = P.wc2_dnorm * P.hi2;
    P.half_hinv = 0.5 * P.h_inv;
    P.alpha_c = P.alpha * P.c;
    P.visc_k = P.alpha_c * P.visc_h;
    P.visc_k2 = 2.0 * P.visc_k;
    P.visc_k2s = P.visc_k2 * P.sg_c;
    P.diff2 = 2.0 * P.diff_coef;

    Phys32& Q = h->phys32;
    const float h32 = (float)P.h;
    Q.cs = (float)h->grid.cs;
    Q.h_inv = 1.0f / h32;
    Q.two_h = 2.0f * h32;
    Q.sr2 = Q.two_h * Q.two_h;
    Q.almostzero = std::sqrt(std::nextafter(Q.sr2, INFINITY) - Q.sr2);
    Q.hi2 = Q.h_inv * Q.h_inv;
    Q.wc2_norm = (c.ndims == 2) ? (float)(7.0 / (4.0 * pi)) * (Q.h_inv * Q.h_inv)
                                : (float)(21.0 / (16.0 * pi)) * ((Q.h_inv * Q.h_inv) * Q.h_inv);
    Q.wc2_dnorm = -5.0f * Q.wc2_norm;
    Q.rho0 = (float)P.rho0;
    Q.B = (float)P.B;
    Q.gamma = (float)P.gamma;
    Q.inv_gamma = (float)P.inv_gamma;
    Q.p_bg = (float)P.p_bg;
    Q.fluid_clip = P.fluid_clip;
    Q.wall_clip = P.wall_clip;
    Q.visc = P.visc;
    Q.diff = P.diff;
    Q.beta = (float)P.beta;
    Q.visc_h = (float)P.visc_h;
    Q.visc_eps_h2 = (float)P.visc_eps_h2;
    Q.visc_ac = (float)(P.alpha * P.c);
    Q.diff_coef = (float)P.diff_coef;
    for (int d = 0; d < 3; ++d) Q.g[d] = (float)P.g[d];
    Q.p_off = (float)P.p_off;
    Q.sg_c = Q.wc2_dnorm * Q.hi2;
    Q.half_hinv = 0.5f * Q.h_inv;
    Q.visc_k = Q.visc_ac * Q.visc_h;
    Q.diff2 = 2.0f * Q.diff_coef;
    Q.az2 = std::nextafter(Q.sr2, INFINITY) - Q.sr2;
    Q.gamma7 = P.gamma == 7.0;
    Q.inv_rho0 = 1.0f / Q.rho0;
}

bool setup_grid(tp_handle* h, std::string& msg) {
    const tp_config& c = h->cfg;
    GridDesc& g = h->grid;
    g.nd = c.ndims;
    g.cs = 2.0 * c.smoothing_length;
    long long total = 1;
    for (int d = 0; d < 3; ++d) {
        if (d < c.ndims) {
            const double lo = std::floor(c.min_corner[d] / g.cs) - 1.0;
            const double hi = std::floor(c.max_corner[d] / g.cs) + 1.0;
            if (!(std::fabs(lo) < 1e9 && std::fabs(hi) < 1e9)) {
                msg = "bounding box too large for the cell size";
                return false;
            }
            g.cmin[d] = (int)lo;
            g.n[d] = (int)(hi - lo) + 1;
        } else {
            g.cmin[d] = 0;
            g.n[d] = 1;
        }
        total *= g.n[d];
        if (total >= (1LL << 30)) {
            msg = "cell grid larger than 2^30 cells";
            return false;
        }
    }
    g.ncells = (int)total;
    return true;
}


// Counting sort of `n` particles with coordinates `u` into key/tmp/start (no packing yet).
// `gate`: device rebuild gate (null = always).  `maxcell`: if non-null, receives (atomicMax) the
// largest cell occupancy of this sort.
tp_status sort_particles(tp_handle* h, const double* u, int n, int* key, int* tmp, int* start,
                         const unsigned* gate = nullptr, int* maxcell = nullptr,
                         bool lex = false) {
    if (!gate) {
        h->lists_owner = 0;  // an unconditional sort replaces the reusable lists
        h->records_order = 0;
    }
    if (n > 0) {
        if (lex) {
            if (h->cfg.ndims == 2)
                k_cell_keys<2, true><<<nblk(n, 256), 256, 0, h->stream>>>(u, n, h->grid, key,
                                                                           h->f_count, h->d_err);
            else
                k_cell_keys<3, true><<<nblk(n, 256), 256, 0, h->stream>>>(u, n, h->grid, key,
                                                                           h->f_count, h->d_err);
        } else if (h->cfg.ndims == 2)
            k_cell_keys<2><<<std::min(nblk(n, 256), 8 * h->num_sms), 256, 0, h->stream>>>(
                u, n, h->grid, key, h->f_count, h->d_err, gate);
        else
            k_cell_keys<3><<<std::min(nblk(n, 256), 8 * h->num_sms), 256, 0, h->stream>>>(
                u, n, h->grid, key, h->f_count, h->d_err, gate);
        TP_LAUNCHED(h, "cell keys");
        h->launches += 1;
        TP_DBG(h, "cell keys");
        if (maxcell) {
            k_max_count<<<256, 256, 0, h->stream>>>(h->f_count, h->grid.ncells, maxcell);
            TP_LAUNCHED(h, "max cell count");
            h->launches += 1;
        }
    }
    const int nc = h->grid.ncells;
    const int nb = nblk(nc, kScanTile);
    const int grid = std::min(nb, 2 * h->num_sms);  // 1024-thread blocks walk the tiles
    k_scan_reduce<<<grid, kScanThreads, 0, h->stream>>>(h->f_count, nc, h->scan_partial, gate);
    k_scan_partials<<<1, kScanThreads, 0, h->stream>>>(h->scan_partial, nb, gate);
    k_scan_final<<<grid, kScanThreads, 0, h->stream>>>(h->f_count, nc, h->scan_partial, start,
                                                     h->f_cursor, gate);
    TP_LAUNCHED(h, "cell scan");
    h->launches += 3;
    TP_DBG(h, "cell scan");
    if (n > 0) {
        k_scatter<<<std::min(nblk(n, 256), 8 * h->num_sms), 256, 0, h->stream>>>(
            key, n, h->f_cursor, tmp, gate);
        TP_LAUNCHED(h, "cell scatter");
        h->launches += 1;
        TP_DBG(h, "cell scatter");
    }
    return TP_OK;
}

// List capacity for a radius 2h (1 + skin) from the largest cell occupancy: the neighbour count
// is at most (ball volume / cell volume) * occupancy; 30 % margin, rounded to 32.
int list_cap(int nd, double skin, int maxcell) {
    const double q = 1.0 + skin;
    const double ball = (nd == 3) ? (4.0 / 3.0) * 3.141592653589793 * q * q * q
                                  : 3.141592653589793 * q * q;
    const double c = std::ceil(1.3 * ball * (double)std::max(maxcell, 1)) + 32.0;
    return ((int)c + 31) / 32 * 32;
}

// Makes the list buffers large enough for fluid coordinates `u` (one host sync).
tp_status ensure_lists(tp_handle* h, const double* u) {
    const int nf = (int)h->cfg.n_fluid, nw = (int)h->cfg.n_wall;
    TP_CUDA(h, cudaMemsetAsync(h->d_max, 0, sizeof(int), h->stream));
    int maxcell_f = 0;
    if (nf > 0) {
        if (h->cfg.ndims == 2)
            k_cell_keys<2><<<nblk(nf, 256), 256, 0, h->stream>>>(u, nf, h->grid, h->f_key,
                                                                  h->f_count, h->d_err);
        else
            k_cell_keys<3><<<nblk(nf, 256), 256, 0, h->stream>>>(u, nf, h->grid, h->f_key,
                                                                  h->f_count, h->d_err);
        k_max_count<<<256, 256, 0, h->stream>>>(h->f_count, h->grid.ncells, h->d_max);
        TP_LAUNCHED(h, "list sizing");
        h->launches += 2;
        TP_DBG(h, "list sizing");
        TP_CUDA(h, cudaMemsetAsync(h->f_count, 0, (size_t)h->grid.ncells * sizeof(int), h->stream));
        TP_CUDA(h, cudaMemcpyAsync(h->h_err + 1, h->d_max, sizeof(int), cudaMemcpyDeviceToHost,
                                   h->stream));
        TP_CUDA(h, cudaStreamSynchronize(h->stream));
        maxcell_f = h->h_err[1];
    }
    const int nd = h->cfg.ndims;
    const int cff = list_cap(nd, h->skin, maxcell_f);
    const int cfw = list_cap(nd, h->skin, h->maxcell_w);
    const int cwf = cff;
    auto grow = [&](unsigned** buf, int* cap, int want, int n) -> cudaError_t {
        if (*cap >= want && *buf) return cudaSuccess;
        h->lists_owner = 0;  // the lists are re-allocated and must be rebuilt
        if (*buf) cudaFree(*buf);
        *buf = nullptr;
        *cap = 0;
        cudaError_t e = dalloc(buf, (size_t)want * (size_t)std::max(n, 1));
        if (e == cudaSuccess) *cap = want;
        return e;
    };
    TP_CUDA(h, grow(&h->l_ff, &h->cap_ff, cff, nf));
    TP_CUDA(h, grow(&h->l_fw, &h->cap_fw, cfw, nf));
    TP_CUDA(h, grow(&h->l_wf, &h->cap_wf, cwf, nw));
    if (h->cfg.precision == TP_PRECISION_FP64) {
        TP_CUDA(h, grow((unsigned**)&h->e_ff, &h->ecap_ff, cff, nf));
        TP_CUDA(h, grow((unsigned**)&h->e_fw, &h->ecap_fw, cfw, nf));
        TP_CUDA(h, grow((unsigned**)&h->e_wf, &h->ecap_wf, cwf, nw));
        if (!h->ec_ff) TP_CUDA(h, dalloc(&h->ec_ff, (size_t)std::max(nf, 1)));
        if (!h->ec_fw) TP_CUDA(h, dalloc(&h->ec_fw, (size_t)std::max(nf, 1)));
        if (!h->acc) {
            TP_CUDA(h, dalloc(&h->acc, (size_t)std::max(nf, 1) * 4));
            TP_CUDA(h, cudaMemsetAsync(h->acc, 0, (size_t)std::max(nf, 1) * 4 * sizeof(double),
                                       h->stream));
        }
    }
    if (debug_sync_enabled())
        std::fprintf(stderr, "tp: lists maxcell_f=%d maxcell_w=%d cap ff=%d fw=%d wf=%d nf=%d nw=%d\n",
                     maxcell_f, h->maxcell_w, h->cap_ff, h->cap_fw, h->cap_wf, nf, nw);
    return TP_OK;
}

// (Re)builds the fluid-fluid, fluid-wall and wall-fluid lists at radius 2h (1 + skin), gated.
tp_status build_lists(tp_handle* h, double skin, const unsigned* gate) {
    const int nf = (int)h->cfg.n_fluid, nw = (int)h->cfg.n_wall;
    const double r = 2.0 * h->cfg.smoothing_length * (1.0 + skin);
    const float r2f = (float)(r * r * (1.0 + 1e-5));
    const float cs = (float)h->grid.cs;
    // the search reaches two cells towards faces closer than r_list - cs (1e-5 cs rounding margin)
    const float m = (float)(r - h->grid.cs + 1e-5 * h->grid.cs);
    // the fluid test records {offsets, rho - rho0}: the first half of the FP32 form's 32-byte
    // records (stride 2), the FP64 form's test array
    const bool f32 = h->cfg.precision == TP_PRECISION_FP32;
    const float4* ftest = f32 ? (const float4*)h->f_rec : h->f_test;
    const int fstride = f32 ? 2 : 1;
    auto run = [&](auto ndc) {
        constexpr int ND = decltype(ndc)::value;
        // the tiled FP32 pair pass enumerates its candidates itself: no fluid lists
        const bool fluid_lists = h->pair_mode != TP_PAIR_TILED;
        if (nf > 0 && fluid_lists)
            k_build_fluid_lists<ND><<<std::min(nblk(nf, 128), 8 * h->num_sms), 128, 0,
                                      h->stream>>>(
                h->grid, cs, m, r2f, nf, ftest, fstride, h->f_skey, h->f_start, h->w_test,
                h->w_skey,
                h->w_start,
                h->l_ff, h->c_ff, h->cap_ff, h->l_fw, h->c_fw, h->cap_fw, h->d_err, gate,
                TileQueue{h->tile_ctr});
        if (nw > 0)
            k_build_wall_lists<ND><<<std::min(nblk(nw, 128), 8 * h->num_sms), 128, 0,
                                     h->stream>>>(
                h->grid, cs, m, r2f, nw, h->w_test, h->w_skey, ftest, fstride, h->f_skey,
                h->f_start,
                h->l_wf,
                h->c_wf, h->cap_wf, h->d_err, gate, TileQueue{h->tile_ctr + 2});
    };
    if (h->cfg.ndims == 2)
        run(std::integral_constant<int, 2>{});
    else
        run(std::integral_constant<int, 3>{});
    TP_LAUNCHED(h, "list build");
    h->launches += (nf > 0 && h->pair_mode != TP_PAIR_TILED) + (nw > 0);
    TP_DBG(h, "list build");
    return TP_OK;
}

// Records the boundary `k` (0..kNumPhases) of the current RHS evaluation's phases.
void mark(tp_handle* h, int k) {
    if (!h->timing) return;
    if (h->ev_used == h->evpool.size()) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) {
            h->timing = false;
            return;
        }
        h->evpool.push_back(e);
    }
    (void)k;
    cudaEventRecord(h->evpool[h->ev_used++], h->stream);
}

void begin_timing(tp_handle* h) {
    h->ev_used = 0;
    for (int k = 0; k < kNumPhases; ++k) h->phase_ms[k] = 0.0;
}

// Sums the phase durations of every RHS evaluation recorded since begin_timing.
void finish_timing(tp_handle* h) {
    if (!h->timing || h->ev_used == 0) return;
    cudaEventSynchronize(h->evpool[h->ev_used - 1]);
    const size_t per = kNumPhases + 1;
    for (size_t b = 0; b + per <= h->ev_used; b += per)
        for (int k = 0; k < kNumPhases; ++k) {
            float ms = 0.0f;
            if (cudaEventElapsedTime(&ms, h->evpool[b + k], h->evpool[b + k + 1]) == cudaSuccess)
                h->phase_ms[k] += ms;
        }
}

tp_status ensure_state(tp_handle* h) {
    if (h->st[0].u) return TP_OK;
    if (!h->x_build) TP_CUDA(h, dalloc(&h->x_build, (size_t)h->cfg.n_fluid * h->cfg.ndims));
    const size_t nf = (size_t)h->cfg.n_fluid;
    const int nd = h->cfg.ndims;
    const bool f32 = h->cfg.precision == TP_PRECISION_FP32;
    for (int k = 0; k < 2; ++k) {
        PhysState& s = h->st[k];
        TP_CUDA(h, dalloc(&s.u, nf * nd));
        TP_CUDA(h, dalloc(&s.tu, nf * nd));
        if (f32) {
            TP_CUDA(h, dalloc((float4**)&s.v, nf));
            TP_CUDA(h, dalloc((float4**)&s.tv, nf));
            TP_CUDA(h, dalloc((float**)&s.m, nf));
        } else {
            TP_CUDA(h, dalloc((double**)&s.v, nf * (nd + 1)));
            TP_CUDA(h, dalloc((double**)&s.tv, nf * (nd + 1)));
            TP_CUDA(h, dalloc((double**)&s.m, nf));
        }
        TP_CUDA(h, dalloc(&s.id, nf));
    }
    return TP_OK;
}

// One RHS evaluation of the cell-sorted pipeline from caller-ordered device arrays:
// sort + pack, exact lists (no skin), Adami.  The pair pass follows in the caller.
tp_status rhs_from_caller(tp_handle* h, const double* u, const double* v) {
    h->lists_owner = 0;  // builds exact-radius lists, which no path can reuse
    const int nf = (int)h->cfg.n_fluid;
    const bool f32 = h->cfg.precision == TP_PRECISION_FP32;
    tp_status st = h->lists_fixed ? TP_OK : ensure_lists(h, u);
    if (st != TP_OK) return st;
    if (!h->x_build) TP_CUDA(h, dalloc(&h->x_build, (size_t)std::max(nf, 1) * h->cfg.ndims));
    mark(h, 0);
    st = sort_particles(h, u, nf, h->f_key, h->f_tmp, h->f_start);
    if (st != TP_OK) return st;
    if (f32)
        fp32_pack(h, u, v, h->m_f, nullptr, nullptr, nullptr);
    else if (nf > 0)
        fp64_pack(h, u, v, h->m_f, nullptr, nullptr, nullptr);
    TP_LAUNCHED(h, "pack");
    h->launches += (nf > 0);
    st = build_lists(h, 0.0, nullptr);
    if (st != TP_OK) return st;
    h->records_order = 1;
    mark(h, 1);
    if (f32)
        fp32_adami(h);
    else
        fp64_adami(h);
    TP_LAUNCHED(h, "adami");
    h->launches += (h->cfg.n_wall > 0);
    mark(h, 2);
    return TP_OK;
}

// The kick! path: the state comes in caller order every call.  Between list rebuilds the slot
// records are refreshed in place from the caller arrays through the permutation of the last
// rebuild and the skin lists are reused; a rebuild (cell sort, stable rank, lists at radius
// 2h (1 + skin)) happens on the device when some particle has moved more than skin * h since
// the last one, or when anything else replaced this handle's cell list.  Pairs are decided
// exactly at every call, so the result equals a fresh neighbour search.
tp_status rhs_kick(tp_handle* h, const double* u, const double* v) {
    const int nf = (int)h->cfg.n_fluid;
    const bool f32 = h->cfg.precision == TP_PRECISION_FP32;
    tp_status st = h->lists_fixed ? TP_OK : ensure_lists(h, u);
    if (st != TP_OK) return st;
    if (!h->x_build) TP_CUDA(h, dalloc(&h->x_build, (size_t)std::max(nf, 1) * h->cfg.ndims));
    const bool force = h->lists_owner != 1;
    h->records_order = 0;
    mark(h, 0);
    k_gate_init<<<1, 32, 0, h->stream>>>(h->gate, (float)(h->skin * h->cfg.smoothing_length),
                                         force ? 1 : 0);
    h->launches += 1;
    if (!force && nf > 0) {
        if (h->cfg.ndims == 2)
            k_displacement<2><<<nblk(nf, 256), 256, 0, h->stream>>>(u, h->x_build, nf, h->gate,
                                                                     h->f_perm);
        else
            k_displacement<3><<<nblk(nf, 256), 256, 0, h->stream>>>(u, h->x_build, nf, h->gate,
                                                                     h->f_perm);
        h->launches += 1;
    }
    st = sort_particles(h, u, nf, h->f_key, h->f_tmp, h->f_start, h->gate);
    if (st != TP_OK) return st;
    if (f32)
        fp32_pack(h, u, v, h->m_f, nullptr, nullptr, h->gate);
    else if (nf > 0)
        fp64_pack(h, u, v, h->m_f, nullptr, nullptr, h->gate);
    TP_LAUNCHED(h, "kick pack");
    h->launches += (nf > 0);
    st = build_lists(h, h->skin, h->gate);
    if (st != TP_OK) return st;
    h->lists_owner = 1;
    h->records_order = 1;
    mark(h, 1);
    if (f32)
        fp32_adami(h);
    else
        fp64_adami(h);
    TP_LAUNCHED(h, "adami");
    h->launches += (h->cfg.n_wall > 0);
    mark(h, 2);
    return TP_OK;
}

}  // namespace

namespace tp {
const double kCK2N54_A[5] = {kA[0], kA[1], kA[2], kA[3], kA[4]};
const double kCK2N54_B[5] = {kB[0], kB[1], kB[2], kB[3], kB[4]};

tp_status api_fail(tp_handle* h, tp_status st, const std::string& msg) { return fail(h, st, msg); }
tp_status api_cuda_fail(tp_handle* h, cudaError_t e, const char* where) {
    return cuda_fail(h, e, where);
}

tp_status sort_fluid_cells(tp_handle* h, const double* u, int* maxcell) {
    const int nf = (int)h->cfg.n_fluid;
    tp_status st = sort_particles(h, u, nf, h->f_key, h->f_tmp, h->f_start, nullptr, maxcell);
    if (st != TP_OK) return st;
    if (nf > 0) {
        k_rank_pack<<<nblk(nf, 256), 256, 0, h->stream>>>(h->f_tmp, h->f_key, h->f_start, nf,
                                                           h->f_perm, h->f_skey, NoPack{},
                                                           nullptr);
        TP_LAUNCHED(h, "rank");
        h->launches += 1;
    }
    return TP_OK;
}
}  // namespace tp

// =========================================================================================
// C ABI
// =========================================================================================
extern "C" {

int32_t tp_abi_version(void) { return TP_ABI_VERSION; }

void tp_config_default(tp_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->ndims = 3;
    c->precision = TP_PRECISION_FP64;
    c->reference_density = 1000.0;
    c->exponent = 7.0;
    c->viscosity_model = TP_VISCOSITY_MONAGHAN;
    c->viscosity_alpha = 0.02;
    c->viscosity_beta = 0.0;
    c->viscosity_epsilon = 0.01;
    c->density_diffusion_model = TP_DIFFUSION_MOLTENI_COLAGROSSI;
    c->density_diffusion_delta = 0.1;
}

tp_status tp_create(const tp_config* cfg, tp_handle** out) {
    if (!out) {
        g_create_error = "null output handle pointer";
        return TP_ERR_ARGUMENT;
    }
    *out = nullptr;
    std::string msg;
    tp_status st = check_config(cfg, msg);
    if (st != TP_OK) {
        g_create_error = msg;
        return st;
    }
    tp_handle* h = new (std::nothrow) tp_handle();
    if (!h) {
        g_create_error = "out of host memory";
        return TP_ERR_CUDA;
    }
    h->cfg = *cfg;
    // measured on GB300 (3D dam break): the FP32 pair kernel runs best with 256-thread blocks
    if (cfg->precision == TP_PRECISION_FP32) h->pair_block = 256;
    if (!setup_grid(h, msg)) {
        g_create_error = msg;
        delete h;
        return TP_ERR_ARGUMENT;
    }
    setup_phys(h);
    const size_t nf = (size_t)cfg->n_fluid, nw = (size_t)cfg->n_wall;
    const size_t nc = (size_t)h->grid.ncells;
    h->scan_blocks = nblk((long)nc, kScanTile);
    cudaError_t e = cudaSuccess;
    auto A = [&](cudaError_t r) {
        if (e == cudaSuccess) e = r;
    };
    A(dalloc(&h->f_key, nf));
    A(dalloc(&h->f_tmp, nf));
    A(dalloc(&h->f_perm, nf));
    A(dalloc(&h->f_skey, nf));
    A(dalloc(&h->f_count, nc));
    A(dalloc(&h->f_start, nc + 1));
    A(dalloc(&h->f_cursor, nc));
    A(dalloc(&h->scan_partial, (size_t)h->scan_blocks));
    A(dalloc(&h->f_test, nf));
    A(dalloc((double4_32a**)&h->f_pos, nf));
    A(dalloc((double4_32a**)&h->f_vel, nf));
    A(dalloc((double4_32a**)&h->f_aux, nf));
    if (cfg->precision == TP_PRECISION_FP32) {
        A(dalloc((double4_32a**)&h->f_rec, nf));
        A(dalloc((double4_32a**)&h->f_rec2, nf));
    }
    A(dalloc(&h->m_f, nf));
    A(dalloc(&h->w_key, nw));
    A(dalloc(&h->w_tmp, nw));
    A(dalloc(&h->w_perm, nw));
    A(dalloc(&h->w_skey, nw));
    A(dalloc(&h->w_start, nc + 1));
    A(dalloc((double4_32a**)&h->w_pos, nw));
    A(dalloc(&h->w_test, nw));
    A(dalloc((double4_32a**)&h->w_state, nw));
    A(dalloc(&h->w_p32, nw));
    A(dalloc(&h->w_vol, nw));
    A(dalloc(&h->c_ff, nf));
    A(dalloc(&h->c_fw, nf));
    A(dalloc(&h->c_wf, nw));
    A(dalloc(&h->gate, 5));
    A(dalloc(&h->tile_ctr, 4));
    A(dalloc(&h->d_max, 1));
    h->red_blocks = 256;
    A(dalloc(&h->red_partial, (size_t)h->red_blocks * 5));
    A(dalloc(&h->d_err, 1));
    A(cudaMallocHost((void**)&h->h_err, 4 * sizeof(int)));
    {
        int dev = 0;
        A(cudaGetDevice(&dev));
        A(cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, dev));
    }
    {
        // the cell origins (cmin + c) * cs32 per axis, computed once here with the FP64 multiply
        // the device would do (exact for cell indices below 2^29: a 24-bit FP32 cell size)
        const GridDesc& g = h->grid;
        const double cs32 = (double)(float)g.cs;
        std::vector<double> org((size_t)(g.n[0] + g.n[1] + g.n[2]));
        size_t k = 0;
        for (int d = 0; d < 3; ++d)
            for (int c = 0; c < g.n[d]; ++c) org[k++] = (double)(g.cmin[d] + c) * cs32;
        A(dalloc(&h->grid_org, org.size()));
        if (e == cudaSuccess)
            e = cudaMemcpy(h->grid_org, org.data(), org.size() * sizeof(double),
                           cudaMemcpyHostToDevice);
        h->grid.org = h->grid_org;
    }
    if (e == cudaSuccess) e = cudaMemset(h->f_count, 0, nc * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(h->d_err, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(h->gate, 0, 5 * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(h->tile_ctr, 0, 4 * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(h->w_start, 0, (nc + 1) * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(h->c_ff, 0, std::max<size_t>(nf, 1) * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(h->c_fw, 0, std::max<size_t>(nf, 1) * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(h->c_wf, 0, std::max<size_t>(nw, 1) * sizeof(int));
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        g_create_error = std::string("device allocation failed: ") + cudaGetErrorString(e);
        tp_destroy(h);
        return TP_ERR_CUDA;
    }
    *out = h;
    return TP_OK;
}

tp_status tp_destroy(tp_handle* h) {
    if (!h) return TP_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    adjoint_release(h);
    void* ptrs[] = {h->f_key,   h->f_tmp,   h->f_perm,  h->f_skey,        h->f_count,
                    h->f_start, h->f_cursor, h->scan_partial, h->f_test, h->f_pos,
                    h->f_vel,   h->f_aux,   h->f_rec,   h->f_rec2,  h->m_f,     h->w_key,
                    h->w_tmp,
                    h->w_perm,  h->w_skey,  h->w_start, h->w_pos,         h->w_test,
                    h->w_state, h->w_p32,   h->w_vol,   h->red_partial, h->d_err};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    void* more[] = {h->l_ff, h->l_fw, h->l_wf, h->c_ff, h->c_fw, h->c_wf, h->x_build, h->gate,
                    h->grid_org, h->tile_ctr,
                    h->d_max, h->e_ff, h->e_fw, h->e_wf, h->ec_ff, h->ec_fw, h->acc, h->spv};
    for (void* p : more)
        if (p) cudaFree(p);
    for (int k = 0; k < 2; ++k) {
        PhysState& s = h->st[k];
        void* q[] = {s.u, s.tu, s.v, s.tv, s.m, s.id};
        for (void* p : q)
            if (p) cudaFree(p);
    }
    if (h->h_err) cudaFreeHost(h->h_err);
    for (cudaEvent_t e : h->evpool) cudaEventDestroy(e);
    delete h;
    return TP_OK;
}

tp_status tp_set_stream(tp_handle* h, void* stream) {
    if (!h) return TP_ERR_ARGUMENT;
    h->stream = (cudaStream_t)stream;
    return TP_OK;
}

tp_status tp_set_wall(tp_handle* h, const double* x_wall, const double* m_wall) {
    if (!h) return TP_ERR_ARGUMENT;
    const int nw = (int)h->cfg.n_wall;
    if (nw > 0 && (!x_wall || !m_wall))
        return fail(h, TP_ERR_ARGUMENT, "tp_set_wall: null coordinates or masses");
    TP_CUDA(h, cudaMemsetAsync(h->d_max, 0, sizeof(int), h->stream));
    tp_status st = sort_particles(h, x_wall, nw, h->w_key, h->w_tmp, h->w_start, nullptr,
                                  h->d_max);
    if (st != TP_OK) return st;
    TP_CUDA(h, cudaMemcpyAsync(h->h_err + 1, h->d_max, sizeof(int), cudaMemcpyDeviceToHost,
                               h->stream));
    TP_CUDA(h, cudaStreamSynchronize(h->stream));
    h->maxcell_w = nw > 0 ? h->h_err[1] : 0;
    if (nw > 0) {
        fp64_pack_wall(h, x_wall, m_wall);
        if (h->cfg.precision == TP_PRECISION_FP32) fp32_init_wall_state(h);
        TP_LAUNCHED(h, "wall pack");
    }
    // A wall particle outside the grid is a configuration error: report it now.
    TP_CUDA(h, cudaMemcpyAsync(h->h_err, h->d_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    TP_CUDA(h, cudaStreamSynchronize(h->stream));
    if (*h->h_err) {
        const int bits = *h->h_err;
        *h->h_err = 0;
        TP_CUDA(h, cudaMemset(h->d_err, 0, sizeof(int)));
        return fail(h, (bits & TP_ERRBIT_NONFINITE) ? TP_ERR_NONFINITE : TP_ERR_OUT_OF_GRID,
                    "tp_set_wall: a wall particle lies outside the FullGridCellList bounds");
    }
    h->wall_set = true;
    return TP_OK;
}

tp_status tp_set_fluid_mass(tp_handle* h, const double* m_fluid) {
    if (!h) return TP_ERR_ARGUMENT;
    const size_t nf = (size_t)h->cfg.n_fluid;
    if (nf > 0 && !m_fluid) return fail(h, TP_ERR_ARGUMENT, "tp_set_fluid_mass: null masses");
    if (nf > 0)
        TP_CUDA(h, cudaMemcpyAsync(h->m_f, m_fluid, nf * sizeof(double), cudaMemcpyDeviceToDevice,
                                   h->stream));
    h->mass_set = true;
    return TP_OK;
}

static tp_status ready(tp_handle* h) {
    if (!h) return TP_ERR_ARGUMENT;
    if (!h->wall_set || !h->mass_set)
        return fail(h, TP_ERR_NOT_READY, "wall geometry (tp_set_wall) and fluid masses "
                                         "(tp_set_fluid_mass) must be set first");
    return TP_OK;
}

tp_status tp_kick(tp_handle* h, double* dv_ode, const double* v_ode, const double* u_ode,
                  double t) {
    (void)t;
    tp_status st = ready(h);
    if (st != TP_OK) return st;
    const int nf = (int)h->cfg.n_fluid;
    if (nf > 0 && (!dv_ode || !v_ode || !u_ode))
        return fail(h, TP_ERR_ARGUMENT, "tp_kick: null array");
    if (nf > 0 && (dv_ode == v_ode || (const double*)dv_ode == u_ode))
        return fail(h, TP_ERR_ARGUMENT, "tp_kick: dv_ode must not alias v_ode or u_ode");
    begin_timing(h);
    st = rhs_kick(h, u_ode, v_ode);
    if (st != TP_OK) return st;
    if (h->cfg.precision == TP_PRECISION_FP32)
        fp32_pair_kick(h, dv_ode);
    else
        fp64_pair_kick(h, dv_ode);
    TP_LAUNCHED(h, "pair");
    h->launches += (nf > 0);
    mark(h, 3);
    finish_timing(h);
    return TP_OK;
}

tp_status tp_sort_particles(tp_handle* h, double* v_ode, double* u_ode, int32_t sort_masses,
                            int32_t* perm_out) {
    tp_status st = ready(h);
    if (st != TP_OK) return st;
    const int nf = (int)h->cfg.n_fluid, nd = h->cfg.ndims;
    if (nf == 0) return TP_OK;
    if (!v_ode || !u_ode) return fail(h, TP_ERR_ARGUMENT, "tp_sort_particles: null array");
    const size_t nv = (size_t)nf * (nd + 1), nu = (size_t)nf * nd;
    if (!h->spv) TP_CUDA(h, dalloc(&h->spv, 2 * nv + nu));  // scratch: v, u, m fit in it
    st = sort_particles(h, u_ode, nf, h->f_key, h->f_tmp, h->f_start, nullptr, nullptr, true);
    if (st != TP_OK) return st;
    k_rank_pack<<<nblk(nf, 256), 256, 0, h->stream>>>(h->f_tmp, h->f_key, h->f_start, nf,
                                                       h->f_perm, h->f_skey, NoPack{}, nullptr);
    double* v2 = h->spv;
    double* u2 = v2 + nv;
    double* m2 = sort_masses ? u2 + nu : nullptr;
    if (nd == 2)
        k_permute_state<2><<<nblk(nf, 256), 256, 0, h->stream>>>(h->f_perm, v_ode, u_ode, h->m_f,
                                                                  v2, u2, m2, nf);
    else
        k_permute_state<3><<<nblk(nf, 256), 256, 0, h->stream>>>(h->f_perm, v_ode, u_ode, h->m_f,
                                                                  v2, u2, m2, nf);
    TP_LAUNCHED(h, "sort particles");
    h->launches += 2;
    TP_CUDA(h, cudaMemcpyAsync(v_ode, v2, nv * sizeof(double), cudaMemcpyDeviceToDevice,
                               h->stream));
    TP_CUDA(h, cudaMemcpyAsync(u_ode, u2, nu * sizeof(double), cudaMemcpyDeviceToDevice,
                               h->stream));
    if (m2)
        TP_CUDA(h, cudaMemcpyAsync(h->m_f, m2, (size_t)nf * sizeof(double),
                                   cudaMemcpyDeviceToDevice, h->stream));
    if (perm_out)
        TP_CUDA(h, cudaMemcpyAsync(perm_out, h->f_perm, (size_t)nf * sizeof(int),
                                   cudaMemcpyDeviceToDevice, h->stream));
    return TP_OK;
}

tp_status tp_integrate_spv(tp_handle* h, double* v_ode, double* u_ode, double t0, double dt,
                           int64_t n_steps) {
    (void)t0;
    tp_status st = ready(h);
    if (st != TP_OK) return st;
    if (n_steps < 0 || !std::isfinite(dt))
        return fail(h, TP_ERR_ARGUMENT, "tp_integrate_spv: bad step count or dt");
    const int nf = (int)h->cfg.n_fluid, nd = h->cfg.ndims;
    if (nf == 0 || n_steps == 0) return TP_OK;
    if (!v_ode || !u_ode) return fail(h, TP_ERR_ARGUMENT, "tp_integrate_spv: null array");
    const size_t nv = (size_t)nf * (nd + 1), nu = (size_t)nf * nd;
    if (!h->spv) TP_CUDA(h, dalloc(&h->spv, 2 * nv + nu));  // k, v_h, u_h
    double* k = h->spv;
    double* vh = k + nv;
    double* uh = vh + nv;
    const double dth = dt * 0.5;
    auto kick = [&](const double* v, const double* u) -> tp_status {
        tp_status s2 = rhs_kick(h, u, v);
        if (s2 != TP_OK) return s2;
        if (h->cfg.precision == TP_PRECISION_FP32)
            fp32_pair_kick(h, k);
        else
            fp64_pair_kick(h, k);
        TP_LAUNCHED(h, "spv kick");
        h->launches += 1;
        return TP_OK;
    };
    for (int64_t step = 0; step < n_steps; ++step) {
        if (nd == 2)
            k_spv_half_drift<2><<<nblk(nf, 256), 256, 0, h->stream>>>(u_ode, v_ode, dth, uh, nf);
        else
            k_spv_half_drift<3><<<nblk(nf, 256), 256, 0, h->stream>>>(u_ode, v_ode, dth, uh, nf);
        st = kick(v_ode, u_ode);
        if (st != TP_OK) return st;
        k_spv_half_kick<<<nblk((long)nv, 256), 256, 0, h->stream>>>(v_ode, k, dth, vh,
                                                                   (long long)nv);
        st = kick(vh, uh);
        if (st != TP_OK) return st;
        if (nd == 2)
            k_spv_finish<2><<<nblk(nf, 256), 256, 0, h->stream>>>(v_ode, u_ode, k, vh, uh, dt,
                                                                   dth, nf);
        else
            k_spv_finish<3><<<nblk(nf, 256), 256, 0, h->stream>>>(v_ode, u_ode, k, vh, uh, dt,
                                                                   dth, nf);
        TP_LAUNCHED(h, "spv update");
        h->launches += 3;
    }
    return TP_OK;
}

tp_status tp_drift(tp_handle* h, double* du_ode, const double* v_ode, const double* u_ode,
                   double t) {
    (void)u_ode;
    (void)t;
    if (!h) return TP_ERR_ARGUMENT;
    const int nf = (int)h->cfg.n_fluid;
    if (nf == 0) return TP_OK;
    if (!du_ode || !v_ode) return fail(h, TP_ERR_ARGUMENT, "tp_drift: null array");
    if (h->cfg.ndims == 2)
        k_drift<2><<<nblk(nf, 256), 256, 0, h->stream>>>(du_ode, v_ode, nf);
    else
        k_drift<3><<<nblk(nf, 256), 256, 0, h->stream>>>(du_ode, v_ode, nf);
    TP_LAUNCHED(h, "drift");
    return TP_OK;
}

}  // extern "C"

namespace tp {

// ---- the fused integrator in pieces (tp_integrate_ck2n54; the batching form's persistent
// capture interleaves the members' stages around one pair launch) ----

// Everything before the first stage: capture checks, state and lists, the caller state loaded
// into slot order, the rebuild gate.  `capturing` receives whether the stream is being captured.
tp_status integrator_begin(tp_handle* h, double* v_ode, double* u_ode, int64_t n_steps,
                           bool* capturing) {
    (void)n_steps;
    tp_status st = TP_OK;
    const int nf = (int)h->cfg.n_fluid, nd = h->cfg.ndims;
    // Under stream capture nothing may synchronise or allocate: list capacities and the
    // integrator state must have been set up by tp_prepare_lists, and timing must be off.
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    TP_CUDA(h, cudaStreamIsCapturing(h->stream, &cap));
    if (cap != cudaStreamCaptureStatusNone && (!h->lists_fixed || !h->st[0].u || h->timing))
        return fail(h, TP_ERR_ARGUMENT,
                    "tp_integrate_ck2n54: capturing needs tp_prepare_lists first and timing off");
    st = ensure_state(h);
    if (st != TP_OK) return st;
    if (!h->lists_fixed) {
        st = ensure_lists(h, u_ode);
        if (st != TP_OK) return st;
    }
    const bool f32 = h->cfg.precision == TP_PRECISION_FP32;
    begin_timing(h);

    // Load the caller state into slot-ordered storage.  Warm start: the lists still belong to
    // the previous call of this integrator, so slot s takes caller particle id[s] of that call's
    // final order and the displacement gate decides about a rebuild.  Cold start (or under
    // capture, so that a graph does not depend on the history): identity order, forced rebuild.
    const bool warm = h->lists_owner == 2 && cap == cudaStreamCaptureStatusNone;
    h->lists_owner = 0;
    h->records_order = 0;
    PhysState& s0 = h->st[h->cur];
    if (warm) {
        auto load = [&](auto ndc, auto f32c) {
            constexpr int ND = decltype(ndc)::value;
            constexpr bool F32 = decltype(f32c)::value;
            k_gather_load<ND, F32><<<nblk(nf, 256), 256, 0, h->stream>>>(
                s0.id, u_ode, v_ode, h->m_f, h->cfg.reference_density, s0.u, s0.v, s0.m, nf);
        };
        if (nd == 2) {
            if (f32) load(std::integral_constant<int, 2>{}, std::true_type{});
            else load(std::integral_constant<int, 2>{}, std::false_type{});
        } else {
            if (f32) load(std::integral_constant<int, 3>{}, std::true_type{});
            else load(std::integral_constant<int, 3>{}, std::false_type{});
        }
        h->launches += 1;
    } else {
        TP_CUDA(h, cudaMemcpyAsync(s0.u, u_ode, (size_t)nf * nd * sizeof(double),
                                   cudaMemcpyDeviceToDevice, h->stream));
        if (f32) {
            if (nd == 2)
                k_load32<2><<<nblk(nf, 256), 256, 0, h->stream>>>(v_ode, h->m_f,
                                                                  h->cfg.reference_density,
                                                                  (float4*)s0.v, (float*)s0.m, nf);
            else
                k_load32<3><<<nblk(nf, 256), 256, 0, h->stream>>>(v_ode, h->m_f,
                                                                  h->cfg.reference_density,
                                                                  (float4*)s0.v, (float*)s0.m, nf);
        } else {
            TP_CUDA(h, cudaMemcpyAsync(s0.v, v_ode, (size_t)nf * (nd + 1) * sizeof(double),
                                       cudaMemcpyDeviceToDevice, h->stream));
            TP_CUDA(h, cudaMemcpyAsync(s0.m, h->m_f, (size_t)nf * sizeof(double),
                                       cudaMemcpyDeviceToDevice, h->stream));
        }
        k_iota<<<nblk(nf, 256), 256, 0, h->stream>>>(s0.id, nf);
        h->launches += f32 ? 2 : 1;
    }
    TP_LAUNCHED(h, "integrator load");
    TP_DBG(h, "integrator load");

    // Rebuild gate (threshold skin * h), forced on a cold start.  Written by a kernel (not a
    // host copy) so that a captured graph carries the values of capture time.
    k_gate_init<<<1, 32, 0, h->stream>>>(h->gate, (float)(h->skin * h->cfg.smoothing_length),
                                         warm ? 0 : 1);
    TP_LAUNCHED(h, "gate init");
    h->launches += 1;

    *capturing = cap != cudaStreamCaptureStatusNone;
    h->rec_prev_fused = false;  // the first stage packs the loaded state
    h->rec_fuse_pending = false;
    return TP_OK;
}

// The stage's displacement check, neighbour search (gated), pack, lists (gated) and Adami pass.
tp_status integrator_stage_pre(tp_handle* h, int64_t step, int stage) {
    tp_status st = TP_OK;
    const int nf = (int)h->cfg.n_fluid, nd = h->cfg.ndims;
    const bool f32 = h->cfg.precision == TP_PRECISION_FP32;
    PhysState& src = h->st[h->cur];
    PhysState& dst = h->st[1 - h->cur];
    mark(h, 0);
    // displacement since the last rebuild (slot order of src = order of x_build): at the
    // first stage of the call a pass over the loaded state; later the previous pair
    // stage has collected it from the positions it wrote (gate[3]), and the advance
    // also consumes the forced flag (the pair kernels read gate[0..2] to know whether
    // this stage moved the state, so none writes them)
    if (step + stage == 0) {
        if (nd == 2)
            k_displacement<2><<<nblk(nf, 256), 256, 0, h->stream>>>(src.u, h->x_build,
                                                                     nf, h->gate);
        else
            k_displacement<3><<<nblk(nf, 256), 256, 0, h->stream>>>(src.u, h->x_build,
                                                                     nf, h->gate);
    } else {
        k_gate_advance<<<1, 32, 0, h->stream>>>(h->gate);
    }
    h->launches += 1;
    TP_DBG(h, "displacement");
    st = sort_particles(h, src.u, nf, h->f_key, h->f_tmp, h->f_start, h->gate);
    if (st != TP_OK) return st;
    if (f32)
        fp32_pack(h, nullptr, nullptr, nullptr, &src, &dst, h->gate, h->rec_prev_fused);
    else
        fp64_pack(h, src.u, (const double*)src.v, (const double*)src.m, &src, &dst,
                  h->gate);
    TP_LAUNCHED(h, "pack");
    h->launches += 1;
    TP_DBG(h, "pack");
    st = build_lists(h, h->skin, h->gate);
    if (st != TP_OK) return st;
    mark(h, 1);
    if (f32)
        fp32_adami(h);
    else
        fp64_adami(h);
    TP_LAUNCHED(h, "adami");
    TP_DBG(h, "adami");
    mark(h, 2);
    return TP_OK;
}

// The stage's pair pass with the fused CK2N54 update; with `desc` (FP32 form) the pass is not
// launched and desc receives it for the batched persistent pass.  In the FP32 list form every
// stage but the call's last also writes the next stage's records (the next pack then runs only
// for a rebuild).
tp_status integrator_stage_pair(tp_handle* h, int stage, double dt, Pair32Member* desc,
                                bool last_stage) {
    const bool f32 = h->cfg.precision == TP_PRECISION_FP32;
    PhysState& src = h->st[h->cur];
    PhysState& dst = h->st[1 - h->cur];
    const bool fuse = f32 && h->pair_mode != TP_PAIR_TILED && !last_stage;
    h->rec_fuse_pending = fuse;
    if (desc) {
        if (!f32) return fail(h, TP_ERR_UNSUPPORTED, "the persistent pair pass is FP32 only");
        fp32_pair_stage(h, src, dst, kA[stage], kB[stage], dt, stage == 0, desc, fuse);
        return TP_OK;
    }
    if (f32)
        fp32_pair_stage(h, src, dst, kA[stage], kB[stage], dt, stage == 0, nullptr, fuse);
    else
        fp64_pair_stage(h, dst, kA[stage], kB[stage], dt, stage == 0);
    return TP_OK;
}

// After the stage's pair pass: bookkeeping and the swap of the ping-pong states.
tp_status integrator_stage_post(tp_handle* h) {
    TP_LAUNCHED(h, "pair stage");
    TP_DBG(h, "pair stage");
    mark(h, 3);
    h->launches += 1 + (h->cfg.n_wall > 0);
    h->cur = 1 - h->cur;
    if (h->rec_fuse_pending) std::swap(h->f_rec, h->f_rec2);  // the records just written
    h->rec_prev_fused = h->rec_fuse_pending;
    h->rec_fuse_pending = false;
    return TP_OK;
}

// After the last stage: the final state back to caller order.
tp_status integrator_end(tp_handle* h, double* v_ode, double* u_ode, bool capturing) {
    const int nf = (int)h->cfg.n_fluid, nd = h->cfg.ndims;
    const bool f32 = h->cfg.precision == TP_PRECISION_FP32;
    const cudaStreamCaptureStatus cap =
        capturing ? cudaStreamCaptureStatusActive : cudaStreamCaptureStatusNone;
    PhysState& sf = h->st[h->cur];
    const double rho0 = h->cfg.reference_density;
    if (nd == 2) {
        if (f32)
            k_store<2, true><<<nblk(nf, 256), 256, 0, h->stream>>>(sf.u, sf.v, sf.id, rho0, u_ode,
                                                                    v_ode, nf);
        else
            k_store<2, false><<<nblk(nf, 256), 256, 0, h->stream>>>(sf.u, sf.v, sf.id, rho0,
                                                                     u_ode, v_ode, nf);
    } else {
        if (f32)
            k_store<3, true><<<nblk(nf, 256), 256, 0, h->stream>>>(sf.u, sf.v, sf.id, rho0, u_ode,
                                                                    v_ode, nf);
        else
            k_store<3, false><<<nblk(nf, 256), 256, 0, h->stream>>>(sf.u, sf.v, sf.id, rho0,
                                                                     u_ode, v_ode, nf);
    }
    TP_LAUNCHED(h, "integrator store");
    TP_DBG(h, "integrator store");
    h->launches += 1;
    // a captured call has not run yet: the next eager call starts cold
    h->lists_owner = cap == cudaStreamCaptureStatusNone ? 2 : 0;
    h->rec_prev_fused = false;
    h->records_order = 2;  // records of the last stage, in the order of the final state
    finish_timing(h);
    return TP_OK;
}

}  // namespace tp

extern "C" {

tp_status tp_integrate_ck2n54(tp_handle* h, double* v_ode, double* u_ode, double t0, double dt,
                              int64_t n_steps) {
    (void)t0;
    tp_status st = ready(h);
    if (st != TP_OK) return st;
    if (n_steps < 0 || !std::isfinite(dt))
        return fail(h, TP_ERR_ARGUMENT, "tp_integrate_ck2n54: bad step count or dt");
    const int nf = (int)h->cfg.n_fluid;
    if (nf == 0 || n_steps == 0) return TP_OK;
    if (!v_ode || !u_ode) return fail(h, TP_ERR_ARGUMENT, "tp_integrate_ck2n54: null array");
    bool capturing = false;
    st = integrator_begin(h, v_ode, u_ode, n_steps, &capturing);
    if (st != TP_OK) return st;
    for (int64_t step = 0; step < n_steps; ++step) {
        for (int stage = 0; stage < 5; ++stage) {
            st = integrator_stage_pre(h, step, stage);
            if (st == TP_OK)
                st = integrator_stage_pair(h, stage, dt, nullptr,
                                           step == n_steps - 1 && stage == 4);
            if (st == TP_OK) st = integrator_stage_post(h);
            if (st != TP_OK) return st;
        }
    }
    return integrator_end(h, v_ode, u_ode, capturing);
}

tp_status tp_fluid_pressure(tp_handle* h, double* p_fluid) {
    if (!h) return TP_ERR_ARGUMENT;
    const int nf = (int)h->cfg.n_fluid;
    if (nf == 0) return TP_OK;
    if (!p_fluid) return fail(h, TP_ERR_ARGUMENT, "tp_fluid_pressure: null array");
    if (h->records_order == 0)
        return fail(h, TP_ERR_NOT_READY,
                    "tp_fluid_pressure: no right-hand side since the particles were last "
                    "reordered (sort, interpolation, adjoint); call tp_kick first");
    const int* ids = h->records_order == 2 ? h->st[h->cur].id : h->f_perm;
    if (h->cfg.precision == TP_PRECISION_FP32)
        fp32_scatter_pressure(h, ids, p_fluid);
    else
        k_scatter_pressure<<<nblk(nf, 256), 256, 0, h->stream>>>((const double4_32a*)h->f_pos,
                                                                 ids, p_fluid, nf);
    TP_LAUNCHED(h, "fluid pressure");
    return TP_OK;
}

tp_status tp_wall_state(tp_handle* h, double* p_wall, double* rho_wall, double* volume_wall) {
    if (!h) return TP_ERR_ARGUMENT;
    const int nw = (int)h->cfg.n_wall;
    if (nw == 0) return TP_OK;
    const double rho0 = h->cfg.reference_density;
    if (h->cfg.precision == TP_PRECISION_FP32)
        k_scatter_wall<true><<<nblk(nw, 256), 256, 0, h->stream>>>(
            h->w_state, h->w_vol, h->w_perm, rho0, p_wall, rho_wall, volume_wall, nw);
    else
        k_scatter_wall<false><<<nblk(nw, 256), 256, 0, h->stream>>>(
            h->w_state, h->w_vol, h->w_perm, rho0, p_wall, rho_wall, volume_wall, nw);
    TP_LAUNCHED(h, "wall state");
    return TP_OK;
}

tp_status tp_div_fast(tp_handle* h, double x64, const double* y64, double* out64, float x32,
                      const float* y32, float* out32, int64_t n) {
    if (!h) return TP_ERR_ARGUMENT;
    if (n < 0 || n > (int64_t)1 << 36)
        return fail(h, TP_ERR_ARGUMENT, "tp_div_fast: bad element count");
    if ((y64 == nullptr) != (out64 == nullptr) || (y32 == nullptr) != (out32 == nullptr))
        return fail(h, TP_ERR_ARGUMENT, "tp_div_fast: an input array without its output");
    if (n == 0 || (!y64 && !y32)) return TP_OK;
    div_fast_check(h, x64, y64, out64, x32, y32, out32, (long long)n);
    TP_LAUNCHED(h, "div_fast");
    return TP_OK;
}

tp_status tp_pair_distance(tp_handle* h, const double* d2, double* r, int64_t n) {
    if (!h) return TP_ERR_ARGUMENT;
    if (n < 0 || n > (int64_t)1 << 36)
        return fail(h, TP_ERR_ARGUMENT, "tp_pair_distance: bad element count");
    if (n == 0) return TP_OK;
    if (!d2 || !r) return fail(h, TP_ERR_ARGUMENT, "tp_pair_distance: null array");
    pair_distance_check(h, d2, r, (long long)n);
    TP_LAUNCHED(h, "pair distance");
    return TP_OK;
}

tp_status tp_nhs_debug(tp_handle* h, const double* u_ode, int32_t* cell, int32_t* order,
                       int32_t* nnb_ff, int32_t* nnb_fw, int32_t* nnb_wf) {
    if (!h) return TP_ERR_ARGUMENT;
    if (!h->wall_set) return fail(h, TP_ERR_NOT_READY, "tp_nhs_debug: wall not set");
    const int nf = (int)h->cfg.n_fluid;
    if (nf > 0 && !u_ode) return fail(h, TP_ERR_ARGUMENT, "tp_nhs_debug: null coordinates");
    tp_status st = sort_particles(h, u_ode, nf, h->f_key, h->f_tmp, h->f_start);
    if (st != TP_OK) return st;
    fp64_pack_pos(h, u_ode);
    TP_LAUNCHED(h, "nhs pack");
    if (cell && nf)
        TP_CUDA(h, cudaMemcpyAsync(cell, h->f_key, (size_t)nf * sizeof(int),
                                   cudaMemcpyDeviceToDevice, h->stream));
    if (order && nf)
        TP_CUDA(h, cudaMemcpyAsync(order, h->f_perm, (size_t)nf * sizeof(int),
                                   cudaMemcpyDeviceToDevice, h->stream));
    fp64_count(h, nnb_ff, nnb_fw, nnb_wf);
    TP_LAUNCHED(h, "neighbour counts");
    return TP_OK;
}

tp_status tp_grid_info(tp_handle* h, int32_t dims[3], double* cell_size, double lo[3]) {
    if (!h) return TP_ERR_ARGUMENT;
    for (int d = 0; d < 3; ++d) {
        if (dims) dims[d] = h->grid.n[d];
        if (lo) lo[d] = (double)h->grid.cmin[d] * h->grid.cs;
    }
    if (cell_size) *cell_size = h->grid.cs;
    return TP_OK;
}

tp_status tp_conservation(tp_handle* h, const double* v_ode, double out[5]) {
    if (!h || !out) return TP_ERR_ARGUMENT;
    const int nf = (int)h->cfg.n_fluid;
    for (int k = 0; k < 5; ++k) out[k] = 0.0;
    if (nf == 0) return TP_OK;
    if (!v_ode) return fail(h, TP_ERR_ARGUMENT, "tp_conservation: null array");
    const int nb = h->red_blocks;
    if (h->cfg.ndims == 2)
        k_conservation<2><<<nb, 256, 0, h->stream>>>(v_ode, h->m_f, nf, h->red_partial);
    else
        k_conservation<3><<<nb, 256, 0, h->stream>>>(v_ode, h->m_f, nf, h->red_partial);
    TP_LAUNCHED(h, "conservation");
    std::vector<double> part((size_t)nb * 5);
    TP_CUDA(h, cudaMemcpyAsync(part.data(), h->red_partial, part.size() * sizeof(double),
                               cudaMemcpyDeviceToHost, h->stream));
    TP_CUDA(h, cudaStreamSynchronize(h->stream));
    // Fixed summation order over the block partials: the result is deterministic.
    for (int b = 0; b < nb; ++b)
        for (int k = 0; k < 5; ++k) out[k] += part[(size_t)b * 5 + k];
    return TP_OK;
}

tp_status tp_sync(tp_handle* h) {
    if (!h) return TP_ERR_ARGUMENT;
    TP_CUDA(h, cudaMemcpyAsync(h->h_err, h->d_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    TP_CUDA(h, cudaStreamSynchronize(h->stream));
    const int bits = *h->h_err;
    if (bits) {
        *h->h_err = 0;
        TP_CUDA(h, cudaMemset(h->d_err, 0, sizeof(int)));
        if (bits & TP_ERRBIT_NONFINITE)
            return fail(h, TP_ERR_NONFINITE, "a particle coordinate became NaN or Inf");
        if (bits & TP_ERRBIT_CAPACITY)
            return fail(h, TP_ERR_CAPACITY,
                        "a neighbour list overflowed its capacity (particles were compressed "
                        "far beyond the densest cell seen when the lists were sized)");
        return fail(h, TP_ERR_OUT_OF_GRID,
                    "a particle left the FullGridCellList bounding box (its cell was clamped)");
    }
    return TP_OK;
}

int32_t tp_phase_times(tp_handle* h, double* ms, int32_t n) {
    if (!h) return 0;
    for (int k = 0; k < n && k < kNumPhases; ++k) ms[k] = h->phase_ms[k];
    return kNumPhases;
}

int64_t tp_kernel_launches(const tp_handle* h) { return h ? (int64_t)h->launches : 0; }

tp_status tp_rebuild_count(tp_handle* h, int64_t* count) {
    if (!h || !count) return TP_ERR_ARGUMENT;
    TP_CUDA(h, cudaMemcpyAsync(h->h_err + 2, h->gate + 4, sizeof(unsigned),
                               cudaMemcpyDeviceToHost, h->stream));
    TP_CUDA(h, cudaStreamSynchronize(h->stream));
    *count = (int64_t)(unsigned)h->h_err[2];
    return TP_OK;
}

tp_status tp_prepare_lists(tp_handle* h, const double* u_ode, double growth) {
    tp_status st = ready(h);
    if (st != TP_OK) return st;
    if (!(growth >= 1.0 && growth <= 16.0))
        return fail(h, TP_ERR_ARGUMENT, "tp_prepare_lists: growth must be in [1, 16]");
    if (h->cfg.n_fluid > 0 && !u_ode) return fail(h, TP_ERR_ARGUMENT, "tp_prepare_lists: null u");
    const double skin = h->skin;
    h->skin = (1.0 + skin) * std::cbrt(growth) - 1.0;  // size for `growth` x the densest cell
    h->lists_fixed = false;
    st = ensure_lists(h, u_ode);
    h->skin = skin;
    if (st != TP_OK) return st;
    st = ensure_state(h);
    if (st != TP_OK) return st;
    h->lists_fixed = true;
    return TP_OK;
}

tp_status tp_interpolate_points(tp_handle* h, const double* v_ode, const double* u_ode,
                                const double* points, int64_t n_points, double smoothing_length,
                                int32_t cut_off_bnd, int32_t clip_negative_pressure,
                                int32_t include_wall_velocity, double* computed_density,
                                double* velocity, double* pressure, double* density,
                                int32_t* neighbor_count) {
    tp_status st = ready(h);
    if (st != TP_OK) return st;
    if (n_points < 0 || !(smoothing_length > 0.0) || !std::isfinite(smoothing_length))
        return fail(h, TP_ERR_ARGUMENT, "tp_interpolate_points: bad point count or smoothing length");
    if (n_points == 0) return TP_OK;
    if (!v_ode || !u_ode || !points || !computed_density || !velocity || !pressure || !density ||
        !neighbor_count)
        return fail(h, TP_ERR_ARGUMENT, "tp_interpolate_points: null array");
    const bool walls = cut_off_bnd || include_wall_velocity;
    // update_systems_and_nhs before the interpolation: cell list of the current fluid state and,
    // when walls take part, their Adami state
    st = walls ? rhs_from_caller(h, u_ode, v_ode) : sort_fluid_cells(h, u_ode, nullptr);
    if (st != TP_OK) return st;
    interp_launch(h, v_ode, u_ode, points, (long long)n_points, smoothing_length, walls,
                  cut_off_bnd != 0, clip_negative_pressure != 0, include_wall_velocity != 0,
                  computed_density, velocity, pressure, density, neighbor_count);
    TP_LAUNCHED(h, "interpolate points");
    return TP_OK;
}

tp_status tp_set_pair_mode(tp_handle* h, int32_t mode) {
    if (!h) return TP_ERR_ARGUMENT;
    if (h->cfg.precision == TP_PRECISION_FP32) {
        if (mode != TP_PAIR_GATHER && mode != TP_PAIR_TILED)
            return fail(h, TP_ERR_ARGUMENT,
                        "the FP32 form's pair mode must be TP_PAIR_GATHER or TP_PAIR_TILED");
    } else if (mode != TP_PAIR_GATHER && mode != TP_PAIR_SYMMETRIC) {
        return fail(h, TP_ERR_ARGUMENT,
                    "the FP64 form's pair mode must be TP_PAIR_GATHER or TP_PAIR_SYMMETRIC");
    }
    // the tiled pass builds no fluid lists: a change of mode hands the lists back
    if (mode != h->pair_mode) h->lists_owner = 0;
    h->pair_mode = mode;
    return TP_OK;
}

tp_status tp_get_config(const tp_handle* h, tp_config* out) {
    if (!h || !out) return TP_ERR_ARGUMENT;
    *out = h->cfg;
    return TP_OK;
}

tp_status tp_set_launch(tp_handle* h, int32_t pair_block) {
    if (!h) return TP_ERR_ARGUMENT;
    if (pair_block != 64 && pair_block != 128 && pair_block != 256)
        return fail(h, TP_ERR_ARGUMENT, "pair_block must be 64, 128 or 256");
    h->pair_block = pair_block;
    return TP_OK;
}

tp_status tp_set_skin(tp_handle* h, double skin) {
    if (!h) return TP_ERR_ARGUMENT;
    if (!(skin >= 0.0 && skin <= 1.0)) return fail(h, TP_ERR_ARGUMENT, "skin must be in [0, 1]");
    if (skin != h->skin) {
        h->lists_fixed = false;  // capacities were sized for the old skin
        h->lists_owner = 0;
    }
    h->skin = skin;
    return TP_OK;
}

tp_status tp_enable_timing(tp_handle* h, int32_t enable) {
    if (!h) return TP_ERR_ARGUMENT;
    h->timing = enable != 0;
    return TP_OK;
}

const char* tp_last_error(const tp_handle* h) {
    if (!h) return g_create_error.c_str();
    return h->last_error.c_str();
}

}  // extern "C"
