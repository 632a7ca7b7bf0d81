// Host side of the batch API declared in include/qhg_gpu.h (qhg_batch_*).
//
// A batch keeps many independent runs of one action list in one device
// table: every run owns a contiguous range of cells (its own grid, neighbour
// indices offset into the range) and therefore a contiguous range of rows of
// the cell-sorted agent table.  One step of the batch is one launch of each
// step kernel over all runs (k_actions, k_cell_scan, k_scatter in their batch
// form, plus k_inject), captured as a CUDA graph per table parity.  Per-run
// values -- seed, step offset, action parameters -- come from a run table in
// device memory; results of a run are the same as those of the run alone.
//
// Admission places a run's grid into a free cell range and stages its agents;
// the next step's cell scan counts them and k_inject writes them after the
// newborns of their cells, so the run's step 0 is the batch step after that.
// Removal clears the run's active flag: its agents leave at the next step and
// its cell range is free after it.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "qhg_device.cuh"
#include "qhg_host.h"
#include "../../include/qhg_gpu.h"

using namespace qhg;

namespace {

thread_local std::string g_batch_error;

int bfail(int code, const std::string &msg) {
    g_batch_error = msg;
    return code;
}

#define BCUDA(expr)                                                                      \
    do {                                                                                 \
        cudaError_t e_ = (expr);                                                         \
        if (e_ != cudaSuccess) {                                                         \
            return bfail(e_ == cudaErrorMemoryAllocation ? QHG_ERR_NOMEM : QHG_ERR_CUDA, \
                         std::string(#expr) + ": " + cudaGetErrorString(e_));            \
        }                                                                                \
    } while (0)

struct RunSlot {
    bool used = false;      // holds a run (active or leaving)
    bool active = false;
    uint32_t cell0 = 0, cell1 = 0;
    int32_t step0 = 0;      // batch step of the run's step 0
    int32_t left_at = -1;   // batch step at which its agents leave (-1: still in)
    bool w_given = false;   // WeightedMove weights given (qhg_batch_set_move_weights), else they follow K
    std::vector<uint8_t> ice;   // the run's ice flags (qhg_batch_set_ice), empty: none
};

}  // namespace

struct qhg_batch {
    qhg_batch_desc desc;
    cudaStream_t stream = nullptr;
    StepConst P;
    LaunchShape shape = {1, 1, 1, 0};
    int nsm = 1, max_ctas_actions = 1, max_ctas_scatter = 1;
    uint32_t cell_cap = 0, agent_cap = 0, stage_cap = 0;
    int max_runs = 0;
    uint32_t cell_hwm = 0;   // cells scanned per step (end of the highest range in use)
    // grid of all runs
    int32_t *d_nbr = nullptr;
    uint8_t *d_nnbr = nullptr;
    uint32_t *d_rev = nullptr;
    double *d_K = nullptr;
    ulonglong2 *d_vthr[2] = {nullptr, nullptr};
    uint64_t *d_wthr = nullptr;
    uint32_t *d_cmove = nullptr;
    uint32_t *d_crun = nullptr;
    // tables (ping-pong)
    int64_t *d_id[2] = {nullptr, nullptr};
    float *d_birth[2] = {nullptr, nullptr};
    float *d_age[2] = {nullptr, nullptr};
    float *d_lastb[2] = {nullptr, nullptr};
    uint8_t *d_meta[2] = {nullptr, nullptr};
    uint32_t *d_ne[2] = {nullptr, nullptr};
    uint32_t *d_necm[2] = {nullptr, nullptr};
    uint32_t *d_nes[2] = {nullptr, nullptr};
    uint32_t *d_tf[2] = {nullptr, nullptr};
    // scratch of a step
    uint32_t *d_outc = nullptr;
    int32_t *d_father = nullptr;
    uint16_t *d_brank = nullptr;
    uint32_t *d_clsc = nullptr, *d_sbase = nullptr, *d_bbase = nullptr, *d_bidb = nullptr, *d_obase = nullptr;
    uint32_t *d_tflag = nullptr;
    uint4 *d_tagg = nullptr, *d_tincl = nullptr;
    // runs
    BatchRun *d_runs = nullptr;
    int64_t *d_rnext = nullptr;
    uint32_t *d_rstat = nullptr;
    // admission
    uint32_t *d_inj = nullptr, *d_ibase = nullptr, *d_injdone = nullptr;
    uint8_t *d_sgender = nullptr;
    unsigned long long *d_stage_err = nullptr;
    uint32_t *d_cstat = nullptr;
    int64_t *d_sid = nullptr;
    float *d_sbirth = nullptr, *d_sage = nullptr, *d_slastb = nullptr;
    uint8_t *d_smeta = nullptr;
    uint32_t *d_scell = nullptr;
    uint32_t staged = 0;            // rows staged for the next step
    // snapshots: cells of the copied rows, a copy stream, and the event that the
    // step after next (which overwrites the copied table) waits for
    uint32_t *d_rowcell = nullptr;
    uint32_t rowcell_cap = 0;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t copy_done = nullptr;
    int32_t copy_table_step = -1;   // batch step after which the copied table is overwritten
    RunState *d_rs = nullptr;
    RunState *h_rs = nullptr;
    int32_t *d_occ = nullptr;   // first occupied step per cell, in each run's steps (when enabled)
    // MoveStats of every run (qhg_batch_move_stats_enable): mode (-1 off), per-cell state,
    // candidates of the step, distances to the neighbour slots
    int32_t ms_mode = -1;
    double ms_radius = 1.0;
    bool ms_cartesian = false;
    int32_t *d_ms_hops = nullptr, *d_ms_chops = nullptr;
    double *d_ms_dist = nullptr, *d_ms_time = nullptr, *d_ms_D = nullptr;
    unsigned long long *d_ms_cdist = nullptr, *d_ms_ckey = nullptr;
    std::vector<RunSlot> slots;
    std::vector<BatchRun> h_runs;
    int32_t gstep = 0;              // batch steps launched
    int cur = 0;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
};

namespace {

void drop_graphs(qhg_batch *b) {
    for (int p = 0; p < 2; p++) {
        if (b->graph[p]) cudaGraphExecDestroy(b->graph[p]);
        b->graph[p] = nullptr;
    }
}

StepBuffers make_buffers(qhg_batch *b, int cur) {
    const int nx = cur ^ 1;
    StepBuffers B;
    memset(&B, 0, sizeof(B));
    B.nonempty = b->d_ne[cur]; B.ne_start = b->d_nes[cur]; B.tile_first = b->d_tf[cur];
    B.id = b->d_id[cur]; B.birth = b->d_birth[cur]; B.age = b->d_age[cur]; B.lastb = b->d_lastb[cur];
    B.meta = b->d_meta[cur];
    B.nonempty2 = b->d_ne[nx]; B.ne_start2 = b->d_nes[nx]; B.tile_first2 = b->d_tf[nx];
    B.id2 = b->d_id[nx]; B.birth2 = b->d_birth[nx]; B.age2 = b->d_age[nx]; B.lastb2 = b->d_lastb[nx];
    B.meta2 = b->d_meta[nx];
    B.nbr = b->d_nbr; B.nnbr = b->d_nnbr; B.rev = b->d_rev; B.K = b->d_K; B.vthr = b->d_vthr[cur]; B.vthr2 = b->d_vthr[nx];
    B.wthr = b->d_wthr; B.cmove = b->d_cmove; B.necm = b->d_necm[cur]; B.necm2 = b->d_necm[nx];
    B.occ = b->d_occ;   // occupation history (qhg_batch_enable_occupancy), else null
    B.ms_mode = b->ms_mode;
    B.ms_hops = b->d_ms_hops; B.ms_dist = b->d_ms_dist; B.ms_time = b->d_ms_time;
    B.ms_chops = b->d_ms_chops; B.ms_cdist = b->d_ms_cdist; B.ms_ckey = b->d_ms_ckey; B.ms_D = b->d_ms_D;
    B.outc = b->d_outc; B.father = b->d_father; B.brank = b->d_brank; B.clsc = b->d_clsc;
    B.sbase = b->d_sbase; B.bbase = b->d_bbase; B.bidbase = b->d_bidb; B.obase = b->d_obase;
    B.tile_flag = b->d_tflag; B.tile_agg = b->d_tagg; B.tile_incl = b->d_tincl;
    return B;
}

BatchBuffers make_batch_buffers(qhg_batch *b) {
    BatchBuffers BB;
    BB.crun = b->d_crun;
    BB.runs = b->d_runs;
    BB.rnext = b->d_rnext;
    BB.rstat = b->d_rstat;
    BB.nruns = b->max_runs;
    BB.inj = b->d_inj;
    BB.ibase = b->d_ibase;
    BB.sid = b->d_sid; BB.sbirth = b->d_sbirth; BB.sage = b->d_sage; BB.slastb = b->d_slastb;
    BB.smeta = b->d_smeta; BB.scell = b->d_scell;
    BB.inj_ctas_done = b->d_injdone;
    BB.cstat = b->d_cstat;
    return BB;
}

// step constants with the cells in use
void refresh_cells(qhg_batch *b) {
    uint32_t hwm = 0;
    for (const RunSlot &s : b->slots) {
        if (s.used) hwm = std::max(hwm, s.cell1);
    }
    hwm = std::max<uint32_t>(hwm, 1u);
    if (hwm != b->cell_hwm) {
        b->cell_hwm = hwm;
        b->P.num_cells = (int32_t)hwm;
        drop_graphs(b);
    }
}

int build_graph(qhg_batch *b, int cur) {
    StepBuffers B = make_buffers(b, cur);
    BatchBuffers BB = make_batch_buffers(b);
    cudaGraph_t g = nullptr;
    BCUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    int le = qhg_launch_step(&b->P, b->d_rs, &B, &BB, &b->shape, b->stream);
    cudaError_t ee = cudaStreamEndCapture(b->stream, &g);
    if (le != 0 || ee != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return bfail(QHG_ERR_CUDA, std::string("graph capture failed: ") +
                                       cudaGetErrorString(le != 0 ? (cudaError_t)le : ee));
    }
    cudaError_t ie = cudaGraphInstantiate(&b->graph[cur], g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) return bfail(QHG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
    return QHG_OK;
}

// reads the run state; a device-side error keeps the last committed step
int pull_state(qhg_batch *b) {
    BCUDA(cudaMemcpyAsync(b->h_rs, b->d_rs, sizeof(RunState), cudaMemcpyDeviceToHost, b->stream));
    BCUDA(cudaStreamSynchronize(b->stream));
    if (b->h_rs->error != 0u) {
        const uint32_t code = b->h_rs->error, info = b->h_rs->error_info;
        // a failed step is not retried: the batch stops at its last committed step
        char buf[160];
        snprintf(buf, sizeof(buf), "device error %u/%u in batch step %d; the batch must be rebuilt", code, info,
                 b->h_rs->step);
        return bfail(code == kErrCellTooLarge ? QHG_ERR_CELL_TOO_LARGE
                     : code == kErrCapacity   ? QHG_ERR_CAPACITY
                     : code == kErrTimeout    ? QHG_ERR_TIMEOUT
                                              : QHG_ERR_DEVICE,
                     buf);
    }
    return QHG_OK;
}

int check_slot(qhg_batch *b, int32_t run) {
    if (run < 0 || run >= b->max_runs || !b->slots[(size_t)run].used) return bfail(QHG_ERR_ARG, "no such run");
    return QHG_OK;
}

}  // namespace

extern "C" const char *qhg_batch_last_error(void) { return g_batch_error.c_str(); }

extern "C" int qhg_batch_create(const qhg_batch_desc *desc, qhg_batch **out) {
    if (desc == nullptr || out == nullptr) return bfail(QHG_ERR_ARG, "null argument");
    if (desc->n_actions < 0 || desc->n_actions > QHG_MAX_ACTIONS) return bfail(QHG_ERR_ARG, "bad n_actions");
    if (desc->max_runs <= 0 || desc->cell_capacity <= 0 || desc->agent_capacity <= 0 || desc->stage_capacity <= 0) {
        return bfail(QHG_ERR_ARG, "capacities must be positive");
    }
    if (desc->agent_capacity > 0x7fffffffLL || desc->cell_capacity > 0x7fffffffLL ||
        desc->stage_capacity > 0x7fffffffLL) {
        return bfail(QHG_ERR_ARG, "capacities above 2^31-1");
    }
    int ndev = 0;
    BCUDA(cudaGetDeviceCount(&ndev));
    if (desc->device < 0 || desc->device >= ndev) return bfail(QHG_ERR_ARG, "bad device ordinal");
    BCUDA(cudaSetDevice(desc->device));
    qhg_batch *b = new qhg_batch();
    b->desc = *desc;
    StepConst &P = b->P;
    memset(&P, 0, sizeof(P));
    // the action list (types and draw windows) is the batch's; parameters are per run
    double zero[QHG_MAX_ACTIONS][4];
    memset(zero, 0, sizeof(zero));
    std::string err;
    if (qhg_host_actions(P, desc->n_actions, desc->action_type, zero, err) != 0) {
        delete b;
        return bfail(QHG_ERR_ARG, err);
    }
    P.n_act = desc->n_actions;
    P.program = qhg_match_program(desc->action_type, desc->n_actions) == 1 ? 1 : 0;
    // a specialised program takes its draws at fixed windows: keep it only if
    // the windows handed out match them
    for (int a = 0; P.program > 0 && a < desc->n_actions; a++) {
        if (P.act[a].window != qhg_program_window(P.program, a)) P.program = 0;
    }
    b->cell_cap = (uint32_t)desc->cell_capacity;
    b->agent_cap = (uint32_t)desc->agent_capacity;
    b->stage_cap = (uint32_t)desc->stage_capacity;
    b->max_runs = desc->max_runs;
    P.capacity = b->agent_cap;
    b->slots.assign((size_t)b->max_runs, RunSlot());
    b->h_runs.assign((size_t)b->max_runs, BatchRun());
    memset(b->h_runs.data(), 0, b->h_runs.size() * sizeof(BatchRun));
    const size_t C = b->cell_cap, N = b->agent_cap, S = b->stage_cap, R = (size_t)b->max_runs;
    const size_t nscan = (C + kScanTile - 1) / kScanTile;
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    auto A = [&](void **p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, bytes);
    };
    A((void **)&b->d_nbr, C * 6 * sizeof(int32_t));
    A((void **)&b->d_nnbr, C);
    A((void **)&b->d_rev, C * sizeof(uint32_t));
    A((void **)&b->d_K, C * sizeof(double));
    A((void **)&b->d_vthr[0], C * sizeof(ulonglong2));
    A((void **)&b->d_vthr[1], C * sizeof(ulonglong2));
    A((void **)&b->d_wthr, C * 6 * sizeof(uint64_t));
    A((void **)&b->d_cmove, C * sizeof(uint32_t));
    A((void **)&b->d_crun, C * sizeof(uint32_t));
    for (int p = 0; p < 2; p++) {
        A((void **)&b->d_id[p], N * sizeof(int64_t) + kColumnPad);
        A((void **)&b->d_birth[p], N * sizeof(float) + kColumnPad);
        A((void **)&b->d_age[p], N * sizeof(float) + kColumnPad);
        A((void **)&b->d_lastb[p], N * sizeof(float) + kColumnPad);
        A((void **)&b->d_meta[p], N + kColumnPad);
        A((void **)&b->d_ne[p], C * sizeof(uint32_t));
        A((void **)&b->d_necm[p], C * sizeof(uint32_t));
        A((void **)&b->d_nes[p], (C + 1) * sizeof(uint32_t));
        A((void **)&b->d_tf[p], (N / kTileAgents + 2) * sizeof(uint32_t));
    }
    A((void **)&b->d_outc, N * sizeof(uint32_t) + kColumnPad);
    A((void **)&b->d_father, N * sizeof(int32_t) + kColumnPad);
    A((void **)&b->d_brank, N * sizeof(uint16_t));
    A((void **)&b->d_clsc, C * kCls * sizeof(uint32_t));
    A((void **)&b->d_sbase, C * sizeof(uint32_t));
    A((void **)&b->d_bbase, C * sizeof(uint32_t));
    A((void **)&b->d_bidb, C * sizeof(uint32_t));
    A((void **)&b->d_obase, C * 6 * sizeof(uint32_t));
    A((void **)&b->d_tflag, nscan * sizeof(uint32_t));
    A((void **)&b->d_tagg, nscan * sizeof(uint4));
    A((void **)&b->d_tincl, nscan * sizeof(uint4));
    A((void **)&b->d_runs, R * sizeof(BatchRun));
    A((void **)&b->d_rnext, R * sizeof(int64_t));
    A((void **)&b->d_rstat, R * kBatchRing * 4 * sizeof(uint32_t));
    A((void **)&b->d_inj, C * sizeof(uint32_t));
    A((void **)&b->d_sgender, S);
    A((void **)&b->d_stage_err, 4 * sizeof(unsigned long long));
    A((void **)&b->d_ibase, C * sizeof(uint32_t));
    A((void **)&b->d_injdone, sizeof(uint32_t));
    A((void **)&b->d_cstat, C * sizeof(uint32_t));
    A((void **)&b->d_sid, S * sizeof(int64_t));
    A((void **)&b->d_sbirth, S * sizeof(float));
    A((void **)&b->d_sage, S * sizeof(float));
    A((void **)&b->d_slastb, S * sizeof(float));
    A((void **)&b->d_smeta, S);
    A((void **)&b->d_scell, S * sizeof(uint32_t));
    A((void **)&b->d_rs, sizeof(RunState));
    if (e == cudaSuccess) e = cudaMallocHost((void **)&b->h_rs, sizeof(RunState));
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_clsc, 0, C * kCls * sizeof(uint32_t), b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_crun, 0xff, C * sizeof(uint32_t), b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_inj, 0, C * sizeof(uint32_t), b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_cstat, 0, C * sizeof(uint32_t), b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_nnbr, 0, C, b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_tflag, 0, nscan * sizeof(uint32_t), b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_injdone, 0, sizeof(uint32_t), b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_rstat, 0, R * kBatchRing * 4 * sizeof(uint32_t), b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_runs, 0, R * sizeof(BatchRun), b->stream);
    if (e == cudaSuccess) {
        // an empty table: no agents, no non-empty cells
        memset(b->h_rs, 0, sizeof(RunState));
        e = cudaMemcpyAsync(b->d_rs, b->h_rs, sizeof(RunState), cudaMemcpyHostToDevice, b->stream);
    }
    const uint32_t zero2[2] = {0u, 0u};
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_nes[0], zero2, sizeof(uint32_t), cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_tf[0], zero2, 2 * sizeof(uint32_t), cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) {
        const std::string msg = std::string("batch create: ") + cudaGetErrorString(e);
        qhg_batch_destroy(b);
        return bfail(e == cudaErrorMemoryAllocation ? QHG_ERR_NOMEM : QHG_ERR_CUDA, msg);
    }
    cudaDeviceGetAttribute(&b->nsm, cudaDevAttrMultiProcessorCount, desc->device);
    b->nsm = std::max(1, b->nsm);
    qhg_tile_ctas_per_sm(&b->max_ctas_actions, &b->max_ctas_scatter);
    b->shape.actions_grid = b->nsm * b->max_ctas_actions;
    b->shape.scatter_grid = b->nsm * b->max_ctas_scatter;
    b->shape.big_grid = b->nsm;
    refresh_cells(b);
    *out = b;
    return QHG_OK;
}

extern "C" int qhg_batch_add_run(qhg_batch *b, const qhg_batch_run_desc *rd, const int32_t *nbr6,
                                 const uint8_t *nnbr, const double *K, int32_t num_cells,
                                 const qhg_agents_soa *a, int64_t n, int32_t *run_out) {
    if (b == nullptr || rd == nullptr || nbr6 == nullptr || nnbr == nullptr || K == nullptr || num_cells <= 0 ||
        run_out == nullptr || n < 0 || (n > 0 && a == nullptr)) {
        return bfail(QHG_ERR_ARG, "bad run arguments");
    }
    if (n > 0 && (a->id == nullptr || a->cell == nullptr || a->birth == nullptr || a->age == nullptr ||
                  a->last_birth == nullptr || a->gender == nullptr || a->state == nullptr)) {
        return bfail(QHG_ERR_ARG, "null agent column");
    }
    BCUDA(cudaSetDevice(b->desc.device));
    // a free run slot; slots of runs that left are reusable once their leaving step has been launched
    int r = -1;
    for (int q = 0; q < b->max_runs; q++) {
        if (!b->slots[(size_t)q].used) { r = q; break; }
    }
    if (r < 0) return bfail(QHG_ERR_CAPACITY, "no free run slot");
    // first free cell range that fits
    const uint32_t C = (uint32_t)num_cells;
    std::vector<std::pair<uint32_t, uint32_t>> used;
    for (const RunSlot &s : b->slots) {
        if (s.used) used.push_back({s.cell0, s.cell1});
    }
    std::sort(used.begin(), used.end());
    uint32_t at = 0;
    bool found = false;
    for (const auto &u : used) {
        if (u.first >= at && u.first - at >= C) { found = true; break; }
        at = std::max(at, u.second);
    }
    if (!found && (uint64_t)at + C <= b->cell_cap) found = true;
    if (!found) return bfail(QHG_ERR_CAPACITY, "no free cell range of that size");
    const uint32_t c0 = at;
    // grid tables of the run, neighbours offset into its range
    std::vector<uint32_t> rev;
    std::vector<uint64_t> wthr;
    std::vector<uint32_t> cmove;
    std::string err;
    if (qhg_host_grid_tables(num_cells, nbr6, nnbr, K, b->P.has_wmove != 0, nullptr, rev, wthr, cmove, err) != 0) {
        return bfail(QHG_ERR_ARG, err);
    }
    std::vector<int32_t> gnbr((size_t)C * 6);
    for (size_t q = 0; q < gnbr.size(); q++) gnbr[q] = nbr6[q] >= 0 ? nbr6[q] + (int32_t)c0 : -1;
    // agents: staged as given; k_batch_stage counts them per cell on the device
    if ((uint64_t)b->staged + (uint64_t)n > b->stage_cap) {
        return bfail(QHG_ERR_CAPACITY, "staging area full: step the batch before admitting more agents");
    }
    const uint32_t s0 = b->staged;
    // the run's constants: its parameters for the batch's action types
    BatchRun R;
    memset(&R, 0, sizeof(R));
    {
        StepConst tmp;
        memset(&tmp, 0, sizeof(tmp));
        if (qhg_host_actions(tmp, b->P.n_act, b->desc.action_type, rd->action_param, err) != 0) {
            return bfail(QHG_ERR_ARG, err);
        }
        for (int q = 0; q < b->P.n_act; q++) R.act[q] = tmp.act[q];
    }
    R.seed = rd->seed;
    R.step0 = b->gstep + 1;
    R.active = 1u;
    R.cell0 = c0;
    R.cell1 = c0 + C;
    cudaStream_t st = b->stream;
    BCUDA(cudaMemcpyAsync(b->d_nbr + (size_t)c0 * 6, gnbr.data(), gnbr.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    BCUDA(cudaMemcpyAsync(b->d_nnbr + c0, nnbr, C, cudaMemcpyHostToDevice, st));
    BCUDA(cudaMemcpyAsync(b->d_rev + c0, rev.data(), C * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    BCUDA(cudaMemcpyAsync(b->d_K + c0, K, C * sizeof(double), cudaMemcpyHostToDevice, st));
    BCUDA(cudaMemcpyAsync(b->d_wthr + (size_t)c0 * 6, wthr.data(), wthr.size() * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
    BCUDA(cudaMemcpyAsync(b->d_cmove + c0, cmove.data(), C * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    std::vector<uint32_t> crun(C, (uint32_t)r);
    BCUDA(cudaMemcpyAsync(b->d_crun + c0, crun.data(), C * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    BCUDA(cudaMemsetAsync(b->d_clsc + (size_t)c0 * kCls, 0, (size_t)C * kCls * sizeof(uint32_t), st));
    BCUDA(cudaMemsetAsync(b->d_inj + c0, 0, C * sizeof(uint32_t), st));
    unsigned long long herr[3] = {0ull, 0ull, ~0ull};   // code, info, largest ID (-1)
    BCUDA(cudaMemcpyAsync(b->d_stage_err, herr, sizeof(herr), cudaMemcpyHostToDevice, st));
    if (n > 0) {
        // the run's rows as given: state in the meta column, gender beside it,
        // cells in the cell column (turned into the batch's cells in place)
        BCUDA(cudaMemcpyAsync(b->d_sid + s0, a->id, n * sizeof(int64_t), cudaMemcpyHostToDevice, st));
        BCUDA(cudaMemcpyAsync(b->d_sbirth + s0, a->birth, n * sizeof(float), cudaMemcpyHostToDevice, st));
        BCUDA(cudaMemcpyAsync(b->d_sage + s0, a->age, n * sizeof(float), cudaMemcpyHostToDevice, st));
        BCUDA(cudaMemcpyAsync(b->d_slastb + s0, a->last_birth, n * sizeof(float), cudaMemcpyHostToDevice, st));
        BCUDA(cudaMemcpyAsync(b->d_smeta + s0, a->state, n, cudaMemcpyHostToDevice, st));
        BCUDA(cudaMemcpyAsync(b->d_sgender + s0, a->gender, n, cudaMemcpyHostToDevice, st));
        BCUDA(cudaMemcpyAsync(b->d_scell + s0, a->cell, n * sizeof(int32_t), cudaMemcpyHostToDevice, st));
        int le = qhg_launch_batch_stage(s0, (uint32_t)n, c0, C, reinterpret_cast<const int32_t *>(b->d_scell + s0),
                                        b->d_smeta, b->d_sgender, b->d_sid, b->d_scell, b->d_inj, b->d_stage_err,
                                        st);
        if (le != 0) return bfail(QHG_ERR_CUDA, std::string("staging: ") + cudaGetErrorString((cudaError_t)le));
    }
    BCUDA(cudaMemcpyAsync(herr, b->d_stage_err, sizeof(herr), cudaMemcpyDeviceToHost, st));
    BCUDA(cudaStreamSynchronize(st));
    if (herr[0] != 0ull) {
        // nothing of the run stays: its cells' counts back to zero
        BCUDA(cudaMemsetAsync(b->d_inj + c0, 0, C * sizeof(uint32_t), st));
        BCUDA(cudaMemsetAsync(b->d_crun + c0, 0xff, C * sizeof(uint32_t), st));
        BCUDA(cudaStreamSynchronize(st));
        if (herr[0] == kErrBadCell) return bfail(QHG_ERR_ARG, "agent cell out of range");
        return bfail(QHG_ERR_CELL_TOO_LARGE, "a cell holds more than QHG_MAX_CELL_AGENTS agents");
    }
    const int64_t nid = (int64_t)herr[2] + 1;
    BCUDA(cudaMemcpyAsync(b->d_runs + r, &R, sizeof(BatchRun), cudaMemcpyHostToDevice, st));
    BCUDA(cudaMemcpyAsync(b->d_rnext + r, &nid, sizeof(int64_t), cudaMemcpyHostToDevice, st));
    BCUDA(cudaMemsetAsync(b->d_rstat + (size_t)r * kBatchRing * 4, 0, kBatchRing * 4 * sizeof(uint32_t), st));
    // the host buffers above are freed on return: wait for the copies
    BCUDA(cudaStreamSynchronize(st));
    b->staged = s0 + (uint32_t)n;
    if (b->d_occ != nullptr) {
        // the run's cells have no entries yet (a leaving run's cells are reused)
        BCUDA(cudaMemsetAsync(b->d_occ + c0, 0xff, C * sizeof(int32_t), st));
    }
    if (b->ms_mode >= 0) {
        // MoveStats of the run: no arrivals yet, distances zero until its
        // coordinates are given; the cells its agents start in are the origins
        std::vector<uint8_t> occupied(C, 0u);
        for (int64_t q = 0; q < n; q++) {
            if (a->state[q] != 0 && a->cell[q] >= 0 && (uint32_t)a->cell[q] < C) occupied[(size_t)a->cell[q]] = 1u;
        }
        std::vector<uint32_t> origin;
        for (uint32_t c = 0; c < C; c++) {
            if (occupied[c]) origin.push_back(c);
        }
        uint32_t *d_origin = nullptr;
        if (!origin.empty()) {
            BCUDA(cudaMalloc(&d_origin, origin.size() * sizeof(uint32_t)));
            BCUDA(cudaMemcpyAsync(d_origin, origin.data(), origin.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
        }
        const int le = qhg_launch_ms_fill(c0, c0 + C, b->ms_mode, d_origin, (uint32_t)origin.size(), b->d_ms_hops,
                                          b->d_ms_dist, b->d_ms_time, b->d_ms_chops, b->d_ms_cdist, b->d_ms_ckey,
                                          b->d_ms_D, st);
        if (le == 0 && d_origin != nullptr) {
            BCUDA(cudaStreamSynchronize(st));
        }
        cudaFree(d_origin);
        if (le != 0) return bfail(QHG_ERR_CUDA, std::string("launch: ") + cudaGetErrorString((cudaError_t)le));
    }
    RunSlot &s = b->slots[(size_t)r];
    s.used = true;
    s.active = true;
    s.w_given = false;
    s.ice.clear();
    s.cell0 = c0;
    s.cell1 = c0 + C;
    s.step0 = R.step0;
    s.left_at = -1;
    b->h_runs[(size_t)r] = R;
    refresh_cells(b);
    *run_out = r;
    return QHG_OK;
}

extern "C" int qhg_batch_remove_run(qhg_batch *b, int32_t run) {
    if (b == nullptr) return bfail(QHG_ERR_ARG, "null batch");
    int rc = check_slot(b, run);
    if (rc != QHG_OK) return rc;
    RunSlot &s = b->slots[(size_t)run];
    if (!s.active) return bfail(QHG_ERR_STATE, "run already removed");
    BCUDA(cudaSetDevice(b->desc.device));
    const uint32_t zero = 0u;
    BCUDA(cudaMemcpyAsync(reinterpret_cast<char *>(b->d_runs + run) + offsetof(BatchRun, active), &zero,
                          sizeof(uint32_t), cudaMemcpyHostToDevice, b->stream));
    BCUDA(cudaStreamSynchronize(b->stream));
    s.active = false;
    s.left_at = b->gstep;   // its agents are dropped by the next step
    b->h_runs[(size_t)run].active = 0u;
    return QHG_OK;
}

// after the leaving step of a run has been launched, its cells belong to no
// run; stream order puts these writes after that step
static int retire_runs(qhg_batch *b) {
    bool changed = false;
    for (size_t q = 0; q < b->slots.size(); q++) {
        RunSlot &s = b->slots[q];
        if (s.used && !s.active && s.left_at >= 0 && b->gstep > s.left_at) {
            BCUDA(cudaMemsetAsync(b->d_crun + s.cell0, 0xff, (size_t)(s.cell1 - s.cell0) * sizeof(uint32_t), b->stream));
            BCUDA(cudaMemsetAsync(b->d_nnbr + s.cell0, 0, (size_t)(s.cell1 - s.cell0), b->stream));
            s.used = false;
            changed = true;
        }
    }
    if (changed) refresh_cells(b);
    return QHG_OK;
}

extern "C" int qhg_batch_step(qhg_batch *b, int32_t nsteps) {
    if (b == nullptr || nsteps < 0) return bfail(QHG_ERR_ARG, "bad step arguments");
    BCUDA(cudaSetDevice(b->desc.device));
    for (int32_t k = 0; k < nsteps; k++) {
        if (b->staged > 0) {
            const uint32_t n = b->staged;
            BCUDA(cudaMemcpyAsync(reinterpret_cast<char *>(b->d_rs) + offsetof(RunState, n_staged), &n,
                                  sizeof(uint32_t), cudaMemcpyHostToDevice, b->stream));
            // the copy reads `n` from this stack frame: wait for it
            BCUDA(cudaStreamSynchronize(b->stream));
        }
        if (b->graph[b->cur] == nullptr) {
            int rc = build_graph(b, b->cur);
            if (rc != QHG_OK) return rc;
        }
        if (b->copy_table_step >= 0 && b->gstep >= b->copy_table_step) {
            // this step writes the table a snapshot is still copying from
            BCUDA(cudaStreamWaitEvent(b->stream, b->copy_done, 0));
            b->copy_table_step = -1;
        }
        BCUDA(cudaGraphLaunch(b->graph[b->cur], b->stream));
        b->cur ^= 1;
        b->gstep++;
        b->staged = 0;
        int rc = retire_runs(b);
        if (rc != QHG_OK) return rc;
    }
    return QHG_OK;
}

extern "C" int qhg_batch_step_timed(qhg_batch *b, int32_t nsteps, float *elapsed_ms) {
    if (b == nullptr || elapsed_ms == nullptr) return bfail(QHG_ERR_ARG, "null argument");
    BCUDA(cudaSetDevice(b->desc.device));
    if (b->ev[0] == nullptr) {
        for (int i = 0; i < 5; i++) BCUDA(cudaEventCreate(&b->ev[i]));
    }
    BCUDA(cudaEventRecord(b->ev[0], b->stream));
    int rc = qhg_batch_step(b, nsteps);
    if (rc != QHG_OK) return rc;
    BCUDA(cudaEventRecord(b->ev[1], b->stream));
    BCUDA(cudaEventSynchronize(b->ev[1]));
    BCUDA(cudaEventElapsedTime(elapsed_ms, b->ev[0], b->ev[1]));
    return pull_state(b);
}

extern "C" int qhg_batch_sync(qhg_batch *b) {
    if (b == nullptr) return bfail(QHG_ERR_ARG, "null batch");
    BCUDA(cudaSetDevice(b->desc.device));
    return pull_state(b);
}

extern "C" int qhg_batch_set_shape(qhg_batch *b, int32_t actions_ctas_per_sm, int32_t scatter_ctas_per_sm) {
    if (b == nullptr) return bfail(QHG_ERR_ARG, "null batch");
    if (actions_ctas_per_sm < 1 || actions_ctas_per_sm > b->max_ctas_actions || scatter_ctas_per_sm < 1 ||
        scatter_ctas_per_sm > b->max_ctas_scatter) {
        return bfail(QHG_ERR_ARG, "CTAs per SM outside what fits");
    }
    b->shape.actions_grid = b->nsm * actions_ctas_per_sm;
    b->shape.scatter_grid = b->nsm * scatter_ctas_per_sm;
    drop_graphs(b);
    return QHG_OK;
}

extern "C" int qhg_batch_get_shape(qhg_batch *b, int32_t *actions_ctas_per_sm, int32_t *scatter_ctas_per_sm,
                                   int32_t *max_actions, int32_t *max_scatter) {
    if (b == nullptr) return bfail(QHG_ERR_ARG, "null batch");
    if (actions_ctas_per_sm) *actions_ctas_per_sm = b->shape.actions_grid / b->nsm;
    if (scatter_ctas_per_sm) *scatter_ctas_per_sm = b->shape.scatter_grid / b->nsm;
    if (max_actions) *max_actions = b->max_ctas_actions;
    if (max_scatter) *max_scatter = b->max_ctas_scatter;
    return QHG_OK;
}

extern "C" int qhg_batch_set_launch(qhg_batch *b, const qhg_batch_launch *l) {
    if (b == nullptr || l == nullptr) return bfail(QHG_ERR_ARG, "null argument");
    if (l->actions_ctas_per_sm < 1 || l->actions_ctas_per_sm > b->max_ctas_actions || l->scatter_ctas_per_sm < 1 ||
        l->scatter_ctas_per_sm > b->max_ctas_scatter) {
        return bfail(QHG_ERR_ARG, "CTAs per SM outside what fits");
    }
    if (l->scan_cells_per_thread < 0 || l->scan_cells_per_thread > 2) {
        return bfail(QHG_ERR_ARG, "scan cells per thread must be 0 (by grid size), 1 or 2");
    }
    if (l->dense_cell < 0 || l->dense_cell > 256) return bfail(QHG_ERR_ARG, "dense_cell must be 0 (default) .. 256");
    int rc = qhg_batch_sync(b);   // the form threshold takes effect at the next commit
    if (rc != QHG_OK) return rc;
    b->shape.actions_grid = b->nsm * l->actions_ctas_per_sm;
    b->shape.scatter_grid = b->nsm * l->scatter_ctas_per_sm;
    b->shape.scan_items = l->scan_cells_per_thread;
    b->P.dense_cell = l->dense_cell > 0 ? (uint32_t)l->dense_cell : kDenseCell;
    drop_graphs(b);
    return QHG_OK;
}

extern "C" int qhg_batch_get_launch(qhg_batch *b, qhg_batch_launch *l) {
    if (b == nullptr || l == nullptr) return bfail(QHG_ERR_ARG, "null argument");
    l->actions_ctas_per_sm = b->shape.actions_grid / b->nsm;
    l->scatter_ctas_per_sm = b->shape.scatter_grid / b->nsm;
    l->scan_cells_per_thread = b->shape.scan_items;
    l->dense_cell = (int32_t)b->P.dense_cell;
    return QHG_OK;
}

extern "C" int qhg_batch_table_info(qhg_batch *b, int64_t *n_agents, int64_t *n_nonempty_cells) {
    if (b == nullptr) return bfail(QHG_ERR_ARG, "null batch");
    int rc = qhg_batch_sync(b);
    if (rc != QHG_OK) return rc;
    if (n_agents) *n_agents = b->h_rs->n_agents;
    if (n_nonempty_cells) *n_nonempty_cells = b->h_rs->n_nonempty;
    return QHG_OK;
}

extern "C" int qhg_batch_run_info(qhg_batch *b, int32_t run, qhg_batch_run_status *info) {
    if (b == nullptr || info == nullptr) return bfail(QHG_ERR_ARG, "null argument");
    int rc = check_slot(b, run);
    if (rc != QHG_OK) return rc;
    const RunSlot &s = b->slots[(size_t)run];
    info->active = s.active ? 1 : 0;
    info->cell0 = (int32_t)s.cell0;
    info->num_cells = (int32_t)(s.cell1 - s.cell0);
    const int32_t end = s.active ? b->gstep : std::min(b->gstep, s.left_at);
    info->steps_done = std::max(0, end - s.step0);
    return QHG_OK;
}

extern "C" int qhg_batch_num_agents(qhg_batch *b, int64_t *n) {
    if (b == nullptr || n == nullptr) return bfail(QHG_ERR_ARG, "null argument");
    int rc = qhg_batch_sync(b);
    if (rc != QHG_OK) return rc;
    *n = b->h_rs->n_agents;
    return QHG_OK;
}

extern "C" int qhg_batch_stats(qhg_batch *b, int32_t run, int32_t nsteps, qhg_step_stats *out) {
    if (b == nullptr || out == nullptr || nsteps < 0 || nsteps > kBatchRing) {
        return bfail(QHG_ERR_ARG, "bad stats arguments (at most 64 steps)");
    }
    int rc = check_slot(b, run);
    if (rc != QHG_OK) return rc;
    rc = qhg_batch_sync(b);
    if (rc != QHG_OK) return rc;
    const RunSlot &s = b->slots[(size_t)run];
    const int32_t end = s.active ? b->gstep : std::min(b->gstep, s.left_at);
    if (end - s.step0 < nsteps) return bfail(QHG_ERR_ARG, "the run has not done that many steps");
    std::vector<uint32_t> ring((size_t)kBatchRing * 4);
    BCUDA(cudaMemcpy(ring.data(), b->d_rstat + (size_t)run * kBatchRing * 4, ring.size() * sizeof(uint32_t),
                     cudaMemcpyDeviceToHost));
    for (int32_t k = 0; k < nsteps; k++) {
        const uint32_t g = (uint32_t)(end - nsteps + k);
        const uint32_t *v = &ring[(size_t)(g % kBatchRing) * 4];
        out[k].live = v[0]; out[k].births = v[1]; out[k].deaths = v[2]; out[k].moves = v[3];
    }
    return QHG_OK;
}

extern "C" int qhg_batch_live_history(qhg_batch *b, int32_t nsteps, uint64_t *live) {
    if (b == nullptr || live == nullptr || nsteps < 0 || nsteps > kStatsRing || nsteps > b->gstep) {
        return bfail(QHG_ERR_ARG, "bad history arguments (at most 1024 steps, at most the steps done)");
    }
    int rc = qhg_batch_sync(b);
    if (rc != QHG_OK) return rc;
    for (int32_t k = 0; k < nsteps; k++) {
        const uint32_t g = (uint32_t)(b->gstep - nsteps + k);
        live[k] = b->h_rs->stats[g % kStatsRing][0];
    }
    return QHG_OK;
}

// rows of a run in the current table: its first row, agents, cell of each row
static int run_rows(qhg_batch *b, int32_t run, uint32_t *row0, uint32_t *count) {
    const RunSlot &s = b->slots[(size_t)run];
    if (!s.active || b->gstep <= s.step0 - 1) return bfail(QHG_ERR_STATE, "the run's agents are not in the table");
    // the last step's scan left each cell's first row in sbase and the run's
    // live count in its statistics slot
    uint32_t r0 = 0, v[4] = {0, 0, 0, 0};
    BCUDA(cudaMemcpy(&r0, b->d_sbase + s.cell0, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    const uint32_t g = (uint32_t)(b->gstep - 1);
    BCUDA(cudaMemcpy(v, b->d_rstat + ((size_t)run * kBatchRing + g % kBatchRing) * 4, sizeof(v),
                     cudaMemcpyDeviceToHost));
    *row0 = r0;
    *count = v[0];
    return QHG_OK;
}

extern "C" int qhg_batch_download(qhg_batch *b, int32_t run, qhg_agents_soa *o, int64_t cap, int64_t *n) {
    if (b == nullptr || o == nullptr || n == nullptr) return bfail(QHG_ERR_ARG, "null argument");
    int rc = check_slot(b, run);
    if (rc != QHG_OK) return rc;
    rc = qhg_batch_sync(b);
    if (rc != QHG_OK) return rc;
    uint32_t row0 = 0, cnt = 0;
    rc = run_rows(b, run, &row0, &cnt);
    if (rc != QHG_OK) return rc;
    *n = cnt;
    if (cap < (int64_t)cnt) return bfail(QHG_ERR_ARG, "output arrays too small");
    if (cnt == 0) return QHG_OK;
    const RunSlot &s = b->slots[(size_t)run];
    const int cur = b->cur;
    uint32_t *d_cell = nullptr;
    BCUDA(cudaMalloc(&d_cell, (size_t)cnt * sizeof(uint32_t)));
    int le = qhg_launch_run_cells(b->d_ne[cur], b->d_nes[cur], b->h_rs->n_nonempty, s.cell0, s.cell1, row0, cnt,
                                  d_cell, nullptr, b->stream);
    cudaError_t e = le == 0 ? cudaStreamSynchronize(b->stream) : (cudaError_t)le;
    std::vector<uint32_t> cells(cnt);
    std::vector<uint8_t> meta(cnt);
    if (e == cudaSuccess) e = cudaMemcpy(cells.data(), d_cell, cnt * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    cudaFree(d_cell);
    if (e == cudaSuccess) e = cudaMemcpy(o->id, b->d_id[cur] + row0, cnt * sizeof(int64_t), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(o->birth, b->d_birth[cur] + row0, cnt * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(o->age, b->d_age[cur] + row0, cnt * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(o->last_birth, b->d_lastb[cur] + row0, cnt * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(meta.data(), b->d_meta[cur] + row0, cnt, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return bfail(QHG_ERR_CUDA, std::string("batch download: ") + cudaGetErrorString(e));
    for (uint32_t i = 0; i < cnt; i++) {
        o->cell[i] = (int32_t)(cells[i] - s.cell0);
        o->gender[i] = meta[i] & kMetaGender;
        o->state[i] = (meta[i] & kMetaFertile) ? QHG_LS_FERTILE : QHG_LS_ALIVE;
    }
    return QHG_OK;
}

extern "C" int qhg_batch_snapshot_async(qhg_batch *b, int32_t run, qhg_agents_soa *o, int64_t cap, int64_t *n,
                                        int32_t *run_step) {
    if (b == nullptr || o == nullptr || n == nullptr) return bfail(QHG_ERR_ARG, "null argument");
    int rc = check_slot(b, run);
    if (rc != QHG_OK) return rc;
    // the table of the last launched step is complete once the stream is idle
    rc = qhg_batch_sync(b);
    if (rc != QHG_OK) return rc;
    uint32_t row0 = 0, cnt = 0;
    rc = run_rows(b, run, &row0, &cnt);
    if (rc != QHG_OK) return rc;
    *n = cnt;
    const RunSlot &s = b->slots[(size_t)run];
    if (run_step) *run_step = b->gstep - s.step0;
    if (cap < (int64_t)cnt) return bfail(QHG_ERR_ARG, "output arrays too small");
    if (b->copy_stream == nullptr) {
        BCUDA(cudaStreamCreateWithFlags(&b->copy_stream, cudaStreamNonBlocking));
        BCUDA(cudaEventCreateWithFlags(&b->copy_done, cudaEventDisableTiming));
    }
    // earlier snapshot copies still use the cell buffer
    BCUDA(cudaStreamSynchronize(b->copy_stream));
    if (cnt > b->rowcell_cap) {
        cudaFree(b->d_rowcell);
        b->d_rowcell = nullptr;
        b->rowcell_cap = 0;
        BCUDA(cudaMalloc(&b->d_rowcell, (size_t)cnt * sizeof(uint32_t)));
        b->rowcell_cap = cnt;
    }
    if (cnt == 0) return QHG_OK;
    const int cur = b->cur;
    cudaStream_t cs = b->copy_stream;
    int le = qhg_launch_run_cells(b->d_ne[cur], b->d_nes[cur], b->h_rs->n_nonempty, s.cell0, s.cell1, row0, cnt,
                                  b->d_rowcell, nullptr, cs);
    if (le != 0) return bfail(QHG_ERR_CUDA, std::string("snapshot cells: ") + cudaGetErrorString((cudaError_t)le));
    // cells as uint32 in the batch's cell space and the meta byte; the caller
    // converts them (cell - cell0, gender = meta & 1, state from meta & 2)
    BCUDA(cudaMemcpyAsync(o->cell, b->d_rowcell, cnt * sizeof(uint32_t), cudaMemcpyDeviceToHost, cs));
    BCUDA(cudaMemcpyAsync(o->id, b->d_id[cur] + row0, cnt * sizeof(int64_t), cudaMemcpyDeviceToHost, cs));
    BCUDA(cudaMemcpyAsync(o->birth, b->d_birth[cur] + row0, cnt * sizeof(float), cudaMemcpyDeviceToHost, cs));
    BCUDA(cudaMemcpyAsync(o->age, b->d_age[cur] + row0, cnt * sizeof(float), cudaMemcpyDeviceToHost, cs));
    BCUDA(cudaMemcpyAsync(o->last_birth, b->d_lastb[cur] + row0, cnt * sizeof(float), cudaMemcpyDeviceToHost, cs));
    BCUDA(cudaMemcpyAsync(o->state, b->d_meta[cur] + row0, cnt, cudaMemcpyDeviceToHost, cs));
    BCUDA(cudaEventRecord(b->copy_done, cs));
    // the next step reads this table, the one after it rewrites it
    b->copy_table_step = b->gstep + 1;
    return QHG_OK;
}

extern "C" int qhg_host_buffer_alloc(int64_t bytes, void **out) {
    if (out == nullptr || bytes < 0) return bfail(QHG_ERR_ARG, "bad buffer arguments");
    *out = nullptr;
    if (bytes == 0) return QHG_OK;
    BCUDA(cudaHostAlloc(out, (size_t)bytes, cudaHostAllocPortable));
    return QHG_OK;
}

extern "C" int qhg_host_buffer_free(void *p) {
    if (p) BCUDA(cudaFreeHost(p));
    return QHG_OK;
}

extern "C" int qhg_batch_snapshot_wait(qhg_batch *b) {
    if (b == nullptr) return bfail(QHG_ERR_ARG, "null batch");
    if (b->copy_stream) BCUDA(cudaStreamSynchronize(b->copy_stream));
    return QHG_OK;
}

extern "C" int qhg_batch_counts(qhg_batch *b, int32_t run, uint32_t *counts) {
    if (b == nullptr || counts == nullptr) return bfail(QHG_ERR_ARG, "null argument");
    int rc = check_slot(b, run);
    if (rc != QHG_OK) return rc;
    rc = qhg_batch_sync(b);
    if (rc != QHG_OK) return rc;
    uint32_t row0 = 0, cnt = 0;
    rc = run_rows(b, run, &row0, &cnt);
    if (rc != QHG_OK) return rc;
    const RunSlot &s = b->slots[(size_t)run];
    const uint32_t C = s.cell1 - s.cell0;
    uint32_t *d_cnt = nullptr;
    BCUDA(cudaMalloc(&d_cnt, (size_t)C * sizeof(uint32_t)));
    cudaError_t e = cudaMemsetAsync(d_cnt, 0, (size_t)C * sizeof(uint32_t), b->stream);
    if (e == cudaSuccess) {
        int le = qhg_launch_run_cells(b->d_ne[b->cur], b->d_nes[b->cur], b->h_rs->n_nonempty, s.cell0, s.cell1, row0,
                                      cnt, nullptr, d_cnt, b->stream);
        e = le == 0 ? cudaStreamSynchronize(b->stream) : (cudaError_t)le;
    }
    if (e == cudaSuccess) e = cudaMemcpy(counts, d_cnt, (size_t)C * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    cudaFree(d_cnt);
    if (e != cudaSuccess) return bfail(QHG_ERR_CUDA, std::string("batch counts: ") + cudaGetErrorString(e));
    return QHG_OK;
}

// ------------------------------------------------- environment of one run
namespace {

// an active run's slot, after the batch's steps so far
int env_slot(qhg_batch *b, int32_t run, RunSlot **out) {
    int rc = check_slot(b, run);
    if (rc != QHG_OK) return rc;
    RunSlot &s = b->slots[(size_t)run];
    if (!s.active) return bfail(QHG_ERR_STATE, "the run has left the batch");
    BCUDA(cudaSetDevice(b->desc.device));
    rc = pull_state(b);
    if (rc != QHG_OK) return rc;
    *out = &s;
    return QHG_OK;
}

// the run's grid as it was admitted: neighbours in its own cell indices,
// neighbour counts, K
int run_grid(qhg_batch *b, const RunSlot &s, std::vector<int32_t> &nbr6, std::vector<uint8_t> &nnbr,
             std::vector<double> &K) {
    const uint32_t C = s.cell1 - s.cell0;
    nbr6.resize((size_t)C * 6);
    nnbr.resize(C);
    K.resize(C);
    BCUDA(cudaMemcpyAsync(nbr6.data(), b->d_nbr + (size_t)s.cell0 * 6, nbr6.size() * sizeof(int32_t),
                          cudaMemcpyDeviceToHost, b->stream));
    BCUDA(cudaMemcpyAsync(nnbr.data(), b->d_nnbr + s.cell0, C, cudaMemcpyDeviceToHost, b->stream));
    BCUDA(cudaMemcpyAsync(K.data(), b->d_K + s.cell0, C * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    BCUDA(cudaStreamSynchronize(b->stream));
    for (int32_t &x : nbr6) x = x >= 0 ? x - (int32_t)s.cell0 : -1;
    return QHG_OK;
}

// the Verhulst thresholds and move words of the run's cells in the current
// table, derived again from K and the move tables (the previous step's cell
// scan derived them from the old ones)
int refresh_run(qhg_batch *b, const RunSlot &s) {
    const int cur = b->cur;
    const uint32_t nne = b->h_rs->n_nonempty;
    if (nne > 0u) {
        const int grid = (int)std::min<uint32_t>((nne + 255u) / 256u, 4096u);
        const int le = qhg_launch_refresh_cells_batch(&b->P, b->d_runs, b->d_crun, b->d_rs, b->d_ne[cur],
                                                      b->d_nes[cur], b->d_K, b->d_cmove, b->d_vthr[cur],
                                                      b->d_necm[cur], s.cell0, s.cell1, grid, b->stream);
        if (le != 0) return bfail(QHG_ERR_CUDA, std::string("launch: ") + cudaGetErrorString((cudaError_t)le));
    }
    BCUDA(cudaStreamSynchronize(b->stream));
    return QHG_OK;
}

int upload_move_tables(qhg_batch *b, const RunSlot &s, const std::vector<uint64_t> &wthr,
                       const std::vector<uint32_t> &cmove) {
    const uint32_t C = s.cell1 - s.cell0;
    BCUDA(cudaMemcpyAsync(b->d_wthr + (size_t)s.cell0 * 6, wthr.data(), (size_t)C * 6 * sizeof(uint64_t),
                          cudaMemcpyHostToDevice, b->stream));
    BCUDA(cudaMemcpyAsync(b->d_cmove + s.cell0, cmove.data(), C * sizeof(uint32_t), cudaMemcpyHostToDevice,
                          b->stream));
    return QHG_OK;
}

}  // namespace

extern "C" int qhg_batch_set_capacity(qhg_batch *b, int32_t run, const double *K) {
    if (b == nullptr || K == nullptr) return bfail(QHG_ERR_ARG, "null argument");
    RunSlot *s = nullptr;
    int rc = env_slot(b, run, &s);
    if (rc != QHG_OK) return rc;
    const uint32_t C = s->cell1 - s->cell0;
    // weights that follow K are derived again (SingleEvaluator over K)
    const bool tables = b->P.has_wmove && !s->w_given;
    std::vector<uint32_t> rev, cmove;
    std::vector<uint64_t> wthr;
    if (tables) {
        std::vector<int32_t> nbr6;
        std::vector<uint8_t> nnbr;
        std::vector<double> oldK;
        rc = run_grid(b, *s, nbr6, nnbr, oldK);
        if (rc != QHG_OK) return rc;
        std::string err;
        if (qhg_host_grid_tables((int)C, nbr6.data(), nnbr.data(), K, true, s->ice.empty() ? nullptr : s->ice.data(),
                                 rev, wthr, cmove, err) != 0) {
            return bfail(QHG_ERR_ARG, err);
        }
    }
    BCUDA(cudaMemcpyAsync(b->d_K + s->cell0, K, C * sizeof(double), cudaMemcpyHostToDevice, b->stream));
    if (tables) {
        rc = upload_move_tables(b, *s, wthr, cmove);
        if (rc != QHG_OK) return rc;
    }
    return refresh_run(b, *s);
}

extern "C" int qhg_batch_set_move_weights(qhg_batch *b, int32_t run, const double *cumw7) {
    if (b == nullptr || cumw7 == nullptr) return bfail(QHG_ERR_ARG, "null argument");
    RunSlot *s = nullptr;
    int rc = env_slot(b, run, &s);
    if (rc != QHG_OK) return rc;
    const uint32_t C = s->cell1 - s->cell0;
    std::vector<int32_t> nbr6;
    std::vector<uint8_t> nnbr;
    std::vector<double> K;
    rc = run_grid(b, *s, nbr6, nnbr, K);
    if (rc != QHG_OK) return rc;
    std::vector<uint32_t> rev, cmove;
    std::vector<uint64_t> wthr;
    {
        std::string err;
        // the neighbour and ice bits of the move words, then the weights' thresholds
        if (qhg_host_grid_tables((int)C, nbr6.data(), nnbr.data(), K.data(), false,
                                 s->ice.empty() ? nullptr : s->ice.data(), rev, wthr, cmove, err) != 0 ||
            qhg_host_move_tables((int)C, nnbr.data(), cumw7, wthr, cmove, err) != 0) {
            return bfail(QHG_ERR_ARG, err);
        }
    }
    rc = upload_move_tables(b, *s, wthr, cmove);
    if (rc != QHG_OK) return rc;
    s->w_given = true;
    return refresh_run(b, *s);
}

extern "C" int qhg_batch_set_ice(qhg_batch *b, int32_t run, const uint8_t *ice) {
    if (b == nullptr) return bfail(QHG_ERR_ARG, "null batch");
    RunSlot *s = nullptr;
    int rc = env_slot(b, run, &s);
    if (rc != QHG_OK) return rc;
    const uint32_t C = s->cell1 - s->cell0;
    std::vector<uint8_t> flags;
    if (ice != nullptr) {
        flags.resize(C);
        for (uint32_t c = 0; c < C; c++) flags[c] = ice[c] != 0 ? 1u : 0u;
    }
    const uint8_t *fp = flags.empty() ? nullptr : flags.data();
    std::vector<int32_t> nbr6;
    std::vector<uint8_t> nnbr;
    std::vector<double> K;
    rc = run_grid(b, *s, nbr6, nnbr, K);
    if (rc != QHG_OK) return rc;
    const bool tables = b->P.has_wmove && !s->w_given;
    if (tables) {
        // weights that follow K give ice cells weight 0
        std::vector<uint32_t> rev, cmove;
        std::vector<uint64_t> wthr;
        std::string err;
        if (qhg_host_grid_tables((int)C, nbr6.data(), nnbr.data(), K.data(), true, fp, rev, wthr, cmove, err) != 0) {
            return bfail(QHG_ERR_ARG, err);
        }
        rc = upload_move_tables(b, *s, wthr, cmove);
        if (rc != QHG_OK) return rc;
    } else {
        // keep the words' other bits (the given weights' all-equal flags)
        std::vector<uint32_t> cur(C);
        BCUDA(cudaMemcpyAsync(cur.data(), b->d_cmove + s->cell0, C * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                              b->stream));
        BCUDA(cudaStreamSynchronize(b->stream));
        qhg_host_ice_bits((int)C, nbr6.data(), fp, cur);
        BCUDA(cudaMemcpyAsync(b->d_cmove + s->cell0, cur.data(), C * sizeof(uint32_t), cudaMemcpyHostToDevice,
                              b->stream));
    }
    s->ice.swap(flags);
    return refresh_run(b, *s);
}

// --------------------------------------------------------------- MoveStats
extern "C" int qhg_batch_move_stats_enable(qhg_batch *b, int32_t mode, double radius, int32_t cartesian) {
    if (b == nullptr) return bfail(QHG_ERR_ARG, "null batch");
    if (mode < QHG_MOVESTATS_FIRST || mode > QHG_MOVESTATS_LAST) return bfail(QHG_ERR_ARG, "bad MoveStats mode");
    if (b->ms_mode >= 0) return bfail(QHG_ERR_STATE, "MoveStats is enabled already");
    for (const RunSlot &s : b->slots) {
        if (s.used) return bfail(QHG_ERR_STATE, "enable MoveStats before the first run is added");
    }
    BCUDA(cudaSetDevice(b->desc.device));
    const size_t C = (size_t)b->cell_cap;
    BCUDA(cudaMalloc((void **)&b->d_ms_hops, C * sizeof(int32_t)));
    BCUDA(cudaMalloc((void **)&b->d_ms_chops, C * sizeof(int32_t)));
    BCUDA(cudaMalloc((void **)&b->d_ms_dist, C * sizeof(double)));
    BCUDA(cudaMalloc((void **)&b->d_ms_time, C * sizeof(double)));
    BCUDA(cudaMalloc((void **)&b->d_ms_D, C * 6 * sizeof(double)));
    BCUDA(cudaMalloc((void **)&b->d_ms_cdist, C * 8));
    BCUDA(cudaMalloc((void **)&b->d_ms_ckey, C * 8));
    const int le = qhg_launch_ms_fill(0u, (uint32_t)C, mode, nullptr, 0u, b->d_ms_hops, b->d_ms_dist, b->d_ms_time,
                                      b->d_ms_chops, b->d_ms_cdist, b->d_ms_ckey, b->d_ms_D, b->stream);
    if (le != 0) return bfail(QHG_ERR_CUDA, std::string("launch: ") + cudaGetErrorString((cudaError_t)le));
    BCUDA(cudaStreamSynchronize(b->stream));
    b->ms_mode = mode;
    b->ms_radius = radius;
    b->ms_cartesian = cartesian != 0;
    drop_graphs(b);   // the step graphs gain the MoveStats kernels
    return QHG_OK;
}

extern "C" int qhg_batch_move_stats_coords(qhg_batch *b, int32_t run, const double *lon, const double *lat) {
    if (b == nullptr || lon == nullptr || lat == nullptr) return bfail(QHG_ERR_ARG, "null argument");
    if (b->ms_mode < 0) return bfail(QHG_ERR_STATE, "MoveStats is not enabled");
    RunSlot *s = nullptr;
    int rc = env_slot(b, run, &s);
    if (rc != QHG_OK) return rc;
    std::vector<int32_t> nbr6;
    std::vector<uint8_t> nnbr;
    std::vector<double> K;
    rc = run_grid(b, *s, nbr6, nnbr, K);
    if (rc != QHG_OK) return rc;
    const uint32_t C = s->cell1 - s->cell0;
    std::vector<double> D((size_t)C * 6, 0.0);
    for (uint32_t c = 0; c < C; c++) {
        for (int k = 0; k < (int)nnbr[c]; k++) {
            const int d = nbr6[(size_t)c * 6 + k];
            if (d >= 0) D[(size_t)c * 6 + k] = qhg_host_move_distance(lon, lat, b->ms_radius, b->ms_cartesian, (int)c, d);
        }
    }
    BCUDA(cudaMemcpyAsync(b->d_ms_D + (size_t)s->cell0 * 6, D.data(), D.size() * sizeof(double), cudaMemcpyHostToDevice,
                          b->stream));
    BCUDA(cudaStreamSynchronize(b->stream));
    return QHG_OK;
}

extern "C" int qhg_batch_move_stats(qhg_batch *b, int32_t run, int32_t *hops, double *dist, double *time) {
    if (b == nullptr || hops == nullptr || dist == nullptr || time == nullptr) return bfail(QHG_ERR_ARG, "null argument");
    if (b->ms_mode < 0) return bfail(QHG_ERR_STATE, "MoveStats is not enabled");
    int rc = check_slot(b, run);
    if (rc != QHG_OK) return rc;
    BCUDA(cudaSetDevice(b->desc.device));
    rc = pull_state(b);
    if (rc != QHG_OK) return rc;
    const RunSlot &s = b->slots[(size_t)run];
    const size_t C = (size_t)(s.cell1 - s.cell0);
    BCUDA(cudaMemcpyAsync(hops, b->d_ms_hops + s.cell0, C * sizeof(int32_t), cudaMemcpyDeviceToHost, b->stream));
    BCUDA(cudaMemcpyAsync(dist, b->d_ms_dist + s.cell0, C * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    BCUDA(cudaMemcpyAsync(time, b->d_ms_time + s.cell0, C * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    BCUDA(cudaStreamSynchronize(b->stream));
    return QHG_OK;
}

// ------------------------------------------------------ occupation history
extern "C" int qhg_batch_enable_occupancy(qhg_batch *b) {
    if (b == nullptr) return bfail(QHG_ERR_ARG, "null batch");
    if (b->d_occ != nullptr) return QHG_OK;
    for (const RunSlot &s : b->slots) {
        if (s.used) return bfail(QHG_ERR_STATE, "enable occupancy tracking before the first run is added");
    }
    BCUDA(cudaSetDevice(b->desc.device));
    BCUDA(cudaMalloc((void **)&b->d_occ, (size_t)b->cell_cap * sizeof(int32_t)));
    BCUDA(cudaMemsetAsync(b->d_occ, 0xff, (size_t)b->cell_cap * sizeof(int32_t), b->stream));
    BCUDA(cudaStreamSynchronize(b->stream));
    drop_graphs(b);   // the step graphs gain the occupancy kernel
    return QHG_OK;
}

extern "C" int qhg_batch_occupancy(qhg_batch *b, int32_t run, int32_t *first_step) {
    if (b == nullptr || first_step == nullptr) return bfail(QHG_ERR_ARG, "null argument");
    if (b->d_occ == nullptr) return bfail(QHG_ERR_STATE, "occupancy tracking is not enabled");
    int rc = check_slot(b, run);
    if (rc != QHG_OK) return rc;
    BCUDA(cudaSetDevice(b->desc.device));
    rc = pull_state(b);
    if (rc != QHG_OK) return rc;
    const RunSlot &s = b->slots[(size_t)run];
    BCUDA(cudaMemcpyAsync(first_step, b->d_occ + s.cell0, (size_t)(s.cell1 - s.cell0) * sizeof(int32_t),
                          cudaMemcpyDeviceToHost, b->stream));
    BCUDA(cudaStreamSynchronize(b->stream));
    return QHG_OK;
}

extern "C" int qhg_batch_stream(qhg_batch *b, void **stream) {
    if (b == nullptr || stream == nullptr) return bfail(QHG_ERR_ARG, "null argument");
    *stream = (void *)b->stream;
    return QHG_OK;
}

extern "C" int qhg_batch_destroy(qhg_batch *b) {
    if (b == nullptr) return QHG_OK;
    cudaSetDevice(b->desc.device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->copy_stream) cudaStreamSynchronize(b->copy_stream);
    drop_graphs(b);
    void *ptrs[] = {b->d_nbr, b->d_nnbr, b->d_rev, b->d_K, b->d_vthr[0], b->d_vthr[1], b->d_wthr, b->d_cmove, b->d_crun,
                    b->d_outc, b->d_father, b->d_brank, b->d_clsc, b->d_sbase, b->d_bbase, b->d_bidb,
                    b->d_obase, b->d_tflag, b->d_tagg, b->d_tincl, b->d_runs, b->d_rnext, b->d_rstat,
                    b->d_inj, b->d_sgender, b->d_stage_err, b->d_ibase, b->d_injdone, b->d_cstat, b->d_sid, b->d_sbirth, b->d_sage,
                    b->d_slastb, b->d_smeta, b->d_scell, b->d_rowcell, b->d_rs, b->d_occ, b->d_ms_hops,
                    b->d_ms_chops, b->d_ms_dist, b->d_ms_time, b->d_ms_D, b->d_ms_cdist, b->d_ms_ckey};
    for (void *p : ptrs) cudaFree(p);
    for (int p = 0; p < 2; p++) {
        cudaFree(b->d_id[p]); cudaFree(b->d_birth[p]); cudaFree(b->d_age[p]); cudaFree(b->d_lastb[p]);
        cudaFree(b->d_meta[p]); cudaFree(b->d_ne[p]); cudaFree(b->d_nes[p]); cudaFree(b->d_tf[p]);
        cudaFree(b->d_necm[p]);
    }
    if (b->h_rs) cudaFreeHost(b->h_rs);
    for (int i = 0; i < 5; i++) {
        if (b->ev[i]) cudaEventDestroy(b->ev[i]);
    }
    if (b->copy_done) cudaEventDestroy(b->copy_done);
    if (b->copy_stream) cudaStreamDestroy(b->copy_stream);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return QHG_OK;
}
