// tp_noalloc.cu — cell sort of the neighbour search for callers that cannot allocate.
//
// Some callers must not allocate device memory themselves or through this library: a host that
// owns every device byte through its own memory pool (a Julia process running CUDA.jl keeps all
// device memory in its pool and its accounting breaks when a foreign library calls cudaMalloc),
// and real-time or fixed-budget loops in which an allocation that can fail or stall mid-run is
// not acceptable.  tp_cell_sort_noalloc gives them the counting sort of the neighbour search
// (cell keys + stable cell-sorted order, the same kernels as the handle path) with every
// scratch array (keys, scatter order, histogram, cursors, cell starts, scan partials, error
// word) carved out of one file-scope device array of fixed size.  The caller passes the
// coordinates and the two output arrays.
//
// The array below is a device symbol: its name in host code is only a host-side stand-in, so
// host code never passes it to a kernel.  Every call looks up its device address with
// cudaGetSymbolAddress in the context that is current at the call (a lookup allocates nothing),
// so a caller that switches contexts (CUDA.jl and other driver-API hosts can make a non-primary
// context current) or resets the device between calls never receives an address of another
// context.  Every call shares the same scratch: the histogram and the error word are cleared at
// the start of each call, everything else is overwritten, and calls that overlap on the GPU (two
// streams, or two host threads) race on the shared scratch and must be serialised by the caller.
// The call is synchronous (it waits for `stream` to read the error word back), so it must not be
// issued while its stream is being captured into a CUDA graph.
#include <cmath>
#include <cstring>

#include "tp_api_internal.h"
#include "tp_nhs.cuh"

namespace {

using namespace tp;

constexpr int kMaxParticles = TP_NOALLOC_MAX_PARTICLES;
constexpr int kMaxCells = TP_NOALLOC_MAX_CELLS;
constexpr int kMaxPartials = (kMaxCells + kScanTile - 1) / kScanTile;
// key, tmp, skey (particles) | count, cursor, start + 1 (cells) | partials | error word
constexpr size_t kScratchInts =
    3 * (size_t)kMaxParticles + 3 * (size_t)kMaxCells + 1 + kMaxPartials + 1;

static __device__ __align__(256) int g_sort_scratch[kScratchInts];

inline int nblk(long n, int t) { return (int)((n + t - 1) / t); }

// Device address of the scratch array in the current context.
cudaError_t scratch_in_current_context(int** out) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_sort_scratch);
    if (e != cudaSuccess) return e;
    *out = (int*)p;
    return cudaSuccess;
}

}  // namespace

extern "C" tp_status tp_cell_sort_noalloc(const tp_config* cfg, const double* u, int64_t n,
                                          int32_t* cell, int32_t* order, void* stream) {
    if (!cfg || (cfg->ndims != 2 && cfg->ndims != 3)) return TP_ERR_ARGUMENT;
    if (n < 0) return TP_ERR_ARGUMENT;
    if (n > kMaxParticles) return TP_ERR_CAPACITY;
    if (n > 0 && (!u || !cell || !order)) return TP_ERR_ARGUMENT;
    if (!(cfg->smoothing_length > 0.0) || !std::isfinite(cfg->smoothing_length))
        return TP_ERR_ARGUMENT;
    // Grid of the neighbour search (same layout as tp_create).
    GridDesc g{};
    g.nd = cfg->ndims;
    g.cs = 2.0 * cfg->smoothing_length;
    long long total = 1;
    for (int d = 0; d < 3; ++d) {
        if (d < g.nd) {
            if (!std::isfinite(cfg->min_corner[d]) || !std::isfinite(cfg->max_corner[d]) ||
                !(cfg->min_corner[d] <= cfg->max_corner[d]))
                return TP_ERR_ARGUMENT;
            const double lo = std::floor(cfg->min_corner[d] / g.cs) - 1.0;
            const double hi = std::floor(cfg->max_corner[d] / g.cs) + 1.0;
            if (!(std::fabs(lo) < 1e9 && std::fabs(hi) < 1e9)) return TP_ERR_CAPACITY;
            g.cmin[d] = (int)lo;
            g.n[d] = (int)(hi - lo) + 1;
        } else {
            g.cmin[d] = 0;
            g.n[d] = 1;
        }
        total *= g.n[d];
        if (total > kMaxCells) return TP_ERR_CAPACITY;
    }
    g.ncells = (int)total;
    if (n == 0) return TP_OK;

    int* base = nullptr;
    if (scratch_in_current_context(&base) != cudaSuccess) return TP_ERR_CUDA;
    int* key = base;
    int* tmp = key + kMaxParticles;
    int* skey = tmp + kMaxParticles;
    int* count = skey + kMaxParticles;
    int* cursor = count + kMaxCells;
    int* start = cursor + kMaxCells;
    int* partial = start + kMaxCells + 1;
    int* err = partial + kMaxPartials;

    cudaStream_t s = (cudaStream_t)stream;
    const int ni = (int)n;
    const int nc = g.ncells;
    const int nb = nblk(nc, kScanTile);
    // The histogram and the error word must start at zero: the previous call may have been cut
    // short, so they are cleared here rather than trusted.
    if (cudaMemsetAsync(count, 0, (size_t)nc * sizeof(int), s) != cudaSuccess) return TP_ERR_CUDA;
    if (cudaMemsetAsync(err, 0, sizeof(int), s) != cudaSuccess) return TP_ERR_CUDA;
    if (g.nd == 2)
        k_cell_keys<2><<<nblk(ni, 256), 256, 0, s>>>(u, ni, g, key, count, err);
    else
        k_cell_keys<3><<<nblk(ni, 256), 256, 0, s>>>(u, ni, g, key, count, err);
    k_scan_reduce<<<nb, kScanThreads, 0, s>>>(count, nc, partial);
    k_scan_partials<<<1, kScanThreads, 0, s>>>(partial, nb);
    k_scan_final<<<nb, kScanThreads, 0, s>>>(count, nc, partial, start, cursor);
    k_scatter<<<nblk(ni, 256), 256, 0, s>>>(key, ni, cursor, tmp);
    k_rank_pack<<<nblk(ni, 256), 256, 0, s>>>(tmp, key, start, ni, order, skey, NoPack{});
    if (cudaGetLastError() != cudaSuccess) return TP_ERR_CUDA;
    if (cudaMemcpyAsync(cell, key, (size_t)ni * sizeof(int), cudaMemcpyDeviceToDevice, s) !=
        cudaSuccess)
        return TP_ERR_CUDA;
    // the error word comes back through a pageable host int: the copy is staged by the driver,
    // and the synchronisation below is what makes `bits` valid to read
    int bits = 0;
    if (cudaMemcpyAsync(&bits, err, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return TP_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return TP_ERR_CUDA;
    if (bits & TP_ERRBIT_NONFINITE) return TP_ERR_NONFINITE;
    if (bits & TP_ERRBIT_OUT_OF_GRID) return TP_ERR_OUT_OF_GRID;
    return TP_OK;
}
