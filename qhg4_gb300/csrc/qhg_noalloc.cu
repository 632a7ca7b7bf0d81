// qhg_gpu_cell_census_noalloc: the per-cell agent census and first rows of a
// cell-sorted table, computed without allocating any memory.
//
// Some callers of this library cannot allocate device memory at the moment
// they need the census: a host runtime that owns a fixed device-memory pool
// and forbids allocations outside it, code that runs while the device heap
// is exhausted, or a real-time loop where an allocation (and the implicit
// device synchronisation of cudaMalloc/cudaFree) is not allowed.  This entry
// point takes the caller's device buffers for its input and outputs and keeps
// its own scratch -- the status words of a decoupled look-back scan -- in a
// file-scope __device__ array of fixed size that every GPU loading the
// library holds until the process exits.
//
// It is a variant of the step's cell scan (k_cell_scan in qhg_kernels.cu):
// the same look-back over tiles of cells, with a single count per cell and
// the tile status words in the static array instead of the run's buffers.
#include <cstdint>
#include <cstring>
#include <string>

#include <cuda_runtime.h>

#include "../../include/qhg_gpu.h"

namespace {

constexpr int kThreads = 256;
constexpr int kItems = 8;
constexpr int kTileCells = kThreads * kItems;
constexpr uint32_t kMaxTiles = (uint32_t)QHG_CENSUS_MAX_CELLS / kTileCells;
constexpr uint32_t kSpinLimit = 1u << 24;

// The scratch shared by every call on a device.  Calls that overlap on the
// GPU race on it; each call leaves its contents behind, and the next call
// resets what has to start at zero (tile counter) or tells stale words apart
// by a per-call epoch (status words).
struct CensusScratch {
    uint32_t tile_counter;
    uint32_t epoch;
    uint32_t error;        // 0 ok, 1 agent cell out of range, 2 look-back gave up
    uint32_t error_info;
    uint32_t flag[kMaxTiles];   // (epoch << 2) | 1 aggregate ready, | 2 inclusive ready
    uint32_t agg[kMaxTiles];
    uint32_t incl[kMaxTiles];
};

static __device__ __align__(256) CensusScratch g_census_scratch;

thread_local std::string g_census_error;

__global__ void k_census_reset(CensusScratch *sc, uint32_t *counts, int C) {
    const int stride = gridDim.x * blockDim.x;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < C; c += stride) counts[c] = 0u;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        sc->tile_counter = 0u;
        sc->error = 0u;
        sc->error_info = 0u;
        sc->epoch = (sc->epoch + 1u) & 0x3fffffffu;
        if (sc->epoch == 0u) sc->epoch = 1u;
    }
}

// per-cell counts by warp-aggregated atomics (lanes of a warp with the same
// cell add together)
__global__ void k_census_count(CensusScratch *sc, const int32_t *cell, int64_t n, int C, uint32_t *counts) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
        const int64_t i = base + threadIdx.x;
        int32_t c = -1;
        if (i < n) c = cell[i];
        const bool ok = (i < n) && c >= 0 && c < C;
        if (i < n && !ok) {
            if (atomicCAS(&sc->error, 0u, 1u) == 0u) sc->error_info = (uint32_t)i;
        }
        const uint32_t key = ok ? (uint32_t)c : 0xffffffffu;
        const uint32_t peers = __match_any_sync(0xffffffffu, key);
        const int leader = __ffs(peers) - 1;
        if (ok && (int)(threadIdx.x & 31) == leader) atomicAdd(&counts[c], (uint32_t)__popc(peers));
    }
}

// exclusive prefix of the counts with a decoupled look-back over tiles of
// kTileCells cells; first_row[C] receives the total
__global__ void __launch_bounds__(kThreads) k_census_scan(CensusScratch *sc, const uint32_t *counts, int C,
                                                          uint32_t *first_row) {
    __shared__ uint32_t s_tile, s_prefix;
    __shared__ uint32_t s_warp[kThreads / 32];
    const uint32_t ntiles = (uint32_t)((C + kTileCells - 1) / kTileCells);
    const uint32_t epoch = sc->epoch;
    if (threadIdx.x == 0) s_tile = atomicAdd(&sc->tile_counter, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile >= ntiles) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int base = (int)tile * kTileCells + threadIdx.x * kItems;
    uint32_t v[kItems];
    uint32_t tot = 0;
#pragma unroll
    for (int j = 0; j < kItems; j++) {
        v[j] = (base + j < C) ? counts[base + j] : 0u;
        tot += v[j];
    }
    uint32_t inc = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t total = 0;
        for (int w = 0; w < kThreads / 32; w++) {
            const uint32_t t = s_warp[w];
            s_warp[w] = total;
            total += t;
        }
        uint32_t excl = 0;
        if (tile == 0) {
            sc->incl[0] = total;
            __threadfence();
            atomicExch(&sc->flag[0], (epoch << 2) | 2u);
        } else {
            sc->agg[tile] = total;
            __threadfence();
            atomicExch(&sc->flag[tile], (epoch << 2) | 1u);
            int t = (int)tile - 1;
            uint32_t spins = 0;
            while (t >= 0) {
                const uint32_t f = atomicAdd(&sc->flag[t], 0u);
                if ((f >> 2) != epoch || (f & 3u) == 0u) {
                    if (++spins > kSpinLimit) {
                        if (atomicCAS(&sc->error, 0u, 2u) == 0u) sc->error_info = tile;
                        break;
                    }
                    continue;
                }
                __threadfence();
                excl += ((f & 3u) == 2u) ? __ldcg(&sc->incl[t]) : __ldcg(&sc->agg[t]);
                if ((f & 3u) == 2u) break;
                t--;
            }
            sc->incl[tile] = excl + total;
            __threadfence();
            atomicExch(&sc->flag[tile], (epoch << 2) | 2u);
        }
        s_prefix = excl;
        if (tile == ntiles - 1) first_row[C] = excl + total;
    }
    __syncthreads();
    uint32_t run = s_prefix + s_warp[warp] + (inc - tot);
#pragma unroll
    for (int j = 0; j < kItems; j++) {
        if (base + j < C) first_row[base + j] = run;
        run += v[j];
    }
}

int census_fail(int code, const std::string &msg) {
    g_census_error = msg;
    return code;
}

}  // namespace

extern "C" const char *qhg_gpu_census_last_error(void) { return g_census_error.c_str(); }

extern "C" int qhg_gpu_cell_census_noalloc(const int32_t *d_agent_cell, int64_t n_agents, int32_t num_cells,
                                           uint32_t *d_counts, uint32_t *d_first_row, void *stream) {
    if (num_cells <= 0 || n_agents < 0 || d_counts == nullptr || d_first_row == nullptr ||
        (n_agents > 0 && d_agent_cell == nullptr)) {
        return census_fail(QHG_ERR_ARG, "bad census arguments");
    }
    if (num_cells > QHG_CENSUS_MAX_CELLS) {
        return census_fail(QHG_ERR_ARG, "num_cells exceeds QHG_CENSUS_MAX_CELLS (" +
                                            std::to_string(QHG_CENSUS_MAX_CELLS) + ")");
    }
    if (n_agents > 0x7fffffffLL) {
        return census_fail(QHG_ERR_ARG, "n_agents exceeds 2^31-1");
    }
    // The device address of the scratch array on the current device.  The
    // array's name in host code is only a host-side stand-in, so the address
    // is looked up with the device current, on every call: a cached address
    // would go stale when the device's context is torn down and rebuilt
    // (cudaDeviceReset), and the lookup allocates nothing.
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_census_scratch);
    if (e != cudaSuccess) {
        return census_fail(QHG_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    }
    CensusScratch *sc = static_cast<CensusScratch *>(p);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int C = num_cells;
    k_census_reset<<<(C + 255) / 256 < 1024 ? (C + 255) / 256 : 1024, 256, 0, st>>>(sc, d_counts, C);
    if (n_agents > 0) {
        int64_t blocks = (n_agents + 255) / 256;
        if (blocks > 4096) blocks = 4096;
        k_census_count<<<(int)blocks, 256, 0, st>>>(sc, d_agent_cell, n_agents, C, d_counts);
    }
    const int ntiles = (C + kTileCells - 1) / kTileCells;
    k_census_scan<<<ntiles, kThreads, 0, st>>>(sc, d_counts, C, d_first_row);
    e = cudaGetLastError();
    if (e != cudaSuccess) return census_fail(QHG_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    uint32_t err[2] = {0u, 0u};
    e = cudaMemcpyAsync(err, &sc->error, sizeof(err), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return census_fail(QHG_ERR_CUDA, std::string("census: ") + cudaGetErrorString(e));
    if (err[0] == 1u) return census_fail(QHG_ERR_ARG, "agent " + std::to_string(err[1]) + " has a cell out of range");
    if (err[0] == 2u) return census_fail(QHG_ERR_TIMEOUT, "census look-back gave up at tile " + std::to_string(err[1]));
    return QHG_OK;
}
