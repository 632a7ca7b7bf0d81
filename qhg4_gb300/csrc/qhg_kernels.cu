// Step kernels of libqhg_gpu.so (sm_103a).
//
// Agents live in device memory as a structure of arrays sorted by cell.
// The non-empty cells are listed in index order (nonempty[r]) together with
// their first row (ne_start[r]).  One step is an action kernel, the cell
// scan and a scatter (plus the genome kernel with genetics).  The action
// kernel and the scatter come in three forms, chosen per step from the table
// the step reads (step_form): warp-per-cell kernels for tables of dense
// cells, cell-aligned tiles for tables of small cells, big-cell tiles when a
// cell holds more than kMaxCell agents.  Every form is launched; the others
// return at once.
//
//   k_actions_cell  one warp per pair of adjacent non-empty cells: the
//                   agents' actions (for a specialised program before the
//                   pairing, both outcomes kept where a mate decides them),
//                   RandomPair (FERTILE members ranked by ID, picks drawn per
//                   picking member and decoded independently), the outcome
//                   word with each agent's rank in its cell's class, the
//                   father's row of each mother, the mothers' birth ranks by
//                   ID with the newborns' genders (in the mothers' outcome
//                   words) and the cells' class counts.
//   k_actions       the same on cell-aligned tiles of ~kTileAgents agents,
//                   one CTA per tile, everything staged in shared memory.
//   k_cell_scan     one pass over all cells with a decoupled look-back scan:
//                   new per-cell counts (stayers + movers in + births), output
//                   bases of every (cell, class), birth numbering, the next
//                   step's non-empty list with first rows, Verhulst
//                   thresholds and move words.
//   k_scatter_cell  one warp per cell, its rows staged in shared memory by
//                   bulk copies: every survivor and newborn written to its
//                   row of the next table, the consumed class counts
//                   cleared.  The last CTA commits.  k_scatter: the tile forms.
//
// The reference runs these as SPopulation::initializeStep / doActions /
// finalizeStep (core/SPopulation.cpp:394-577, 596-724, 1058-1092, 509-536).
#include <algorithm>
#include <climits>
#include <cstring>
#include <cstdint>
#include <cuda_runtime.h>

#include "qhg_device.cuh"

namespace qhg {

#define FULL_MASK 0xffffffffu

__device__ __forceinline__ uint32_t pick4(const Draw4 &d, uint32_t k) {
    const uint32_t a = (k & 1u) ? d.v[1] : d.v[0];
    const uint32_t b = (k & 1u) ? d.v[3] : d.v[2];
    return (k & 2u) ? b : a;
}

// draws of one agent in one step: the per-agent action stream, caching the
// last Philox block.  The first block is drawn at once, where the warp is
// converged (the actions' draws are taken under divergent conditions, and
// most of them fall in that block).
template <bool BATCH>
struct AgentDraws {
    uint64_t seed;
    int64_t id;
    uint32_t step;
    uint32_t blk;
    Draw4 d;
    __device__ __forceinline__ void init(const StepConst &P, uint64_t s, uint32_t st, int64_t i) {
        seed = s; step = st; id = i; blk = kStreamActions;
        d = run_block<BATCH>(P, s, st, i, kStreamActions);
    }
    __device__ __forceinline__ uint32_t get(const StepConst &P, uint32_t k) {
        const uint32_t b = kStreamActions + (k >> 2);
        if (b != blk) {
            d = run_block<BATCH>(P, seed, step, id, b);
            blk = b;
        }
        return pick4(d, k & 3u);
    }
};

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void set_error(RunState *rs, uint32_t code, uint32_t info) {
    if (atomicCAS(&rs->error, 0u, code) == 0u) {
        rs->error_info = info;
    }
}

// u < thr  <=>  u / 2^32 < x   for a double x (the reference's wrandd() < x)
__device__ __forceinline__ uint64_t prob_threshold(double x) {
    if (!(x > 0.0)) return 0ull;
    const double y = __dmul_rn(x, 4294967296.0);
    if (y >= 4294967296.0) return 4294967296ull;
    return (uint64_t)ceil(y);
}

// LinearBirth / LinearDeath ::initialize for one cell holding n agents
// (actions/LinearBirth.cpp:90-112, actions/LinearDeath.cpp:92-122), as
// integer thresholds: x = birth (kind 1) or birth-rate death (kind 2)
// threshold with the kind in bits 62-63, y = death threshold
__device__ __forceinline__ ulonglong2 verhulst_thresholds(const ActionConst &A, double Kcell, uint32_t n) {
    double B, D;
    const double K = (A.type == kVerhulst) ? A.K : Kcell;
    if (A.type == kVerhulstVarK && K <= 0.0) {
        B = 0.0;
        D = 1.0;
    } else {
        const double r = __ddiv_rn((double)n, K);
        B = __dadd_rn(A.b0, __dmul_rn(A.th_b0, r));
        D = __dadd_rn(A.d0, __dmul_rn(A.th_d0, r));
    }
    uint64_t x = 0;
    if (B > 0.0) x = prob_threshold(B) | (1ull << 62);
    else if (B < 0.0) x = prob_threshold(-B) | (2ull << 62);
    return make_ulonglong2(x, prob_threshold(D));
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Warp-aggregated shared-memory counter: lanes with the same key add `unit`
// each to *addr with one atomic per key; every lane gets the old value plus
// unit times its rank within the key.  All 32 lanes must call it (lanes with
// valid == false pass along and get 0).
__device__ __forceinline__ uint32_t warp_agg_add(bool valid, uint32_t key, uint32_t *addr, uint32_t unit) {
    const uint32_t k = valid ? key : 0xffffffffu;
    const uint32_t peers = __match_any_sync(FULL_MASK, k);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if (valid && lane == leader) base = atomicAdd(addr, (uint32_t)__popc(peers) * unit);
    base = __shfl_sync(FULL_MASK, base, leader);
    return valid ? base + (uint32_t)__popc(peers & lanemask_lt()) * unit : 0u;
}

__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t *red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL_MASK, v, o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    uint32_t t = 0;
    if (threadIdx.x == 0) {
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
    }
    return t;
}

// ------------------------------------------------------------------ actions
// Action programs compiled into specialised k_actions kernels.  Program 0
// interprets the run's action list at run time; programs 1-3 are the orders
// of the benchmark populations (ascending priority): 1 Fertility,
// RandomPair, Verhulst, RandomMove, GetOld; 2 Fertility, RandomPair,
// VerhulstVarK, WeightedMove, GetOld, OldAgeDeath; 3 as 1 with VerhulstVarK.
__host__ __device__ constexpr int prog_len(int p) {
    return p == 1 ? 5 : (p == 2 ? 6 : (p == 3 ? 5 : 0));
}
__host__ __device__ constexpr int prog_act(int p, int a) {
    return p == 1 ? (a == 0 ? kFertility : a == 1 ? kRandomPair : a == 2 ? kVerhulst : a == 3 ? kRandomMove : kGetOld)
         : p == 2 ? (a == 0 ? kFertility : a == 1 ? kRandomPair : a == 2 ? kVerhulstVarK : a == 3 ? kWeightedMove
                     : a == 4 ? kGetOld : kOldAgeDeath)
         : p == 3 ? (a == 0 ? kFertility : a == 1 ? kRandomPair : a == 2 ? kVerhulstVarK : a == 3 ? kRandomMove : kGetOld)
         : -1;
}
constexpr int kNumPrograms = 4;

template <int TM, int TT, bool BATCH>
struct ActionsSmemT {
    int64_t fid[TM];         // IDs of the unsorted FERTILE lists (same positions as pick), then of the OldAgeDeath queue
    float ofa[TM];           // ages of the OldAgeDeath queue
    uint16_t cell[TM];       // local cell index of each row
    int16_t mate[TM];        // mate's row within the tile, -1 none
    uint16_t frank[TM];      // rank of a FERTILE agent among its cell's FERTILE agents of its sex (by ID)
    uint16_t list[TM];       // at each cell's rows: FERTILE females by ID, then FERTILE males by ID
    uint16_t pick[TM];       // at each cell's rows: unsorted FERTILE lists (rows), then the mothers' ID ranks
    uint16_t pkpos[TM];      // list positions of the tile's picking members (dense)
    uint16_t oadq[TM];       // list positions of the tile's FERTILE agents (dense), then at each
                             // cell's rows the pick values, then the OldAgeDeath queue (rows)
    uint8_t oc[TM];          // outcome byte
    uint32_t cstart[kTileCells + 1];  // first row of each cell, relative to the tile
    int32_t cid[kTileCells];
    uint32_t crun[BATCH ? kTileCells : 1];   // batches: run of each cell
    uint32_t dm[BATCH ? kTileCells : 1];     // batches: deaths | moves << 16 per cell
    uint32_t nfm[kTileCells];      // FERTILE females | FERTILE males << 16
    uint64_t tb[kTileCells];       // Verhulst: birth threshold (kind 1) or birth-rate death threshold (kind 2)
    uint64_t td[kTileCells];       // LinearDeath threshold
    uint8_t tk[kTileCells];
    uint8_t nn[kTileCells];        // moves: neighbours of each cell
    uint8_t vm[kTileCells];        // moves: bit q set when neighbour slot q holds a cell
    uint8_t wv[kTileCells];        // WeightedMove: bit q set when neighbour slot q holds a cell that is not ice
    uint8_t wf[kTileCells];        // WeightedMove: all weights of the cell equal
    uint32_t cls[kTileCells][4];   // class counts, two 16-bit counters per word
    uint32_t red[TT / 32];
    uint32_t npick, noad, nfert, idhi;
};

// OldAgeDeath is the last action of program 2: its draw (needed only by
// agents whose age lies inside the death window) is made in a dense pass
// after the other actions, so that warps do not run Philox for a few lanes
__host__ __device__ constexpr bool prog_defers_oad(int p) { return p == 2; }
// position of OldAgeDeath in a specialised program, -1 if it has none
__host__ __device__ constexpr int prog_oad_index(int p) {
    return p == 0 ? -1 : (prog_act(p, 0) == kOldAgeDeath ? 0 : prog_act(p, 1) == kOldAgeDeath ? 1
                          : prog_act(p, 2) == kOldAgeDeath ? 2 : prog_act(p, 3) == kOldAgeDeath ? 3
                          : prog_act(p, 4) == kOldAgeDeath ? 4 : prog_act(p, 5) == kOldAgeDeath ? 5 : -1);
}
// position of an action type in a specialised program (-1 if absent); for
// Verhulst either of its two forms, for moves either of the two move actions
__host__ __device__ constexpr int prog_index(int p, int t0, int t1) {
    return p == 0 ? -1 : (prog_act(p, 0) == t0 || prog_act(p, 0) == t1 ? 0
                          : prog_act(p, 1) == t0 || prog_act(p, 1) == t1 ? 1
                          : prog_act(p, 2) == t0 || prog_act(p, 2) == t1 ? 2
                          : prog_act(p, 3) == t0 || prog_act(p, 3) == t1 ? 3
                          : prog_act(p, 4) == t0 || prog_act(p, 4) == t1 ? 4
                          : prog_act(p, 5) == t0 || prog_act(p, 5) == t1 ? 5 : -1);
}
// draws an action takes from the agent's action stream, and the first draw
// (window) of action a of a specialised program: windows follow execution
// order, as the host hands them out
__host__ __device__ constexpr uint32_t action_draws(int t) {
    return (t == kVerhulst || t == kVerhulstVarK || t == kRandomMove || t == kWeightedMove) ? 2u
           : (t == kOldAgeDeath || t == kATanDeath ? 1u : 0u);
}
__host__ __device__ constexpr uint32_t prog_window(int p, int a) {
    return a <= 0 ? 0u : prog_window(p, a - 1) + action_draws(prog_act(p, a - 1));
}
// how agent_outcome treats an agent inside the OldAgeDeath window: draw and
// decide, leave it to the caller (queued), or apply a decision made before
constexpr int kOadDraw = 0, kOadQueue = 1, kOadGiven = 2;

// Rank of an agent's outcome in its cell's class (slot 0 stay, 1..6 movers
// per neighbour slot) from a warp-aggregated shared counter; every lane of
// the warp calls it.  The rank is the agent's offset in the class: rows of a
// cell are not kept in ID order, and nothing depends on their order.
__device__ __forceinline__ uint32_t class_rank(bool counted, int lc, int cls, uint32_t (*cnt)[4]) {
    const int slot = (cls > 0) ? cls - 1 : 0;
    const uint32_t q = warp_agg_add(counted, ((uint32_t)lc << 3) | (uint32_t)slot, &cnt[lc][slot >> 1],
                                    1u << (16 * (slot & 1)));
    return (q >> (16 * (slot & 1))) & 0xffffu;
}

// cell constants one agent's actions read
struct CellView {
    uint64_t tb, td;      // Verhulst: birth (kind 1) or birth-rate death (kind 2) threshold, death threshold
    uint32_t tk;          // Verhulst kind (0 none)
    uint32_t nn, vm, wf;  // moves: neighbour count, valid neighbour slots, all weights equal
    uint32_t wv;          // WeightedMove: valid neighbour slots that are not ice
    uint32_t c;           // cell index (WeightedMove thresholds)
};

// Every action of one agent in execution order (SPopulation::doActions,
// core/SPopulation.cpp:554-577; GetOld actions/GetOld.cpp:37-48, Fertility
// actions/Fertility.cpp:49-73, LinearBirth/LinearDeath actions/LinearBirth.cpp:122-166,
// actions/LinearDeath.cpp:131-150, OldAgeDeath actions/OldAgeDeath.cpp:48-67,
// RandomMove actions/RandomMove.cpp:65-100, WeightedMove actions/WeightedMove.cpp:45-106).
// Returns the outcome byte.  An agent inside the OldAgeDeath window draws
// (OAD == kOadDraw), is left alive with `queued` set for the caller to draw
// (kOadQueue), or dies as `oad_die` says (kOadGiven).
// `fa` is the agent's age after the actions (the input age on entry);
// `mdir` the direction of the move it registered (neighbour slot + 1, 0
// none), also when a later action killed it.
template <int PROG, bool BATCH, int OAD>
__device__ __forceinline__ uint8_t agent_outcome(const StepConst &P, const BatchRun *R, int32_t step, float fT,
                                                 int64_t id, uint8_t m8, float fb, float fa_in, float fl,
                                                 bool mated, const CellView &cv, const uint64_t *__restrict__ wthr,
                                                 bool oad_die, float &fa, bool &queued, uint32_t &cnt_deaths,
                                                 uint32_t &cnt_moves, uint32_t &mdir) {
    const uint64_t seed = BATCH ? R->seed : P.seed;
    const int32_t stepR = BATCH ? step - R->step0 : step;
    const float fTR = BATCH ? (float)stepR : fT;
    fa = fa_in;
    const bool female = !(m8 & kMetaGender);
    bool fert = (m8 & kMetaFertile) != 0;
    bool alive = true;
    bool bflag = false;
    int dir = 0;
    AgentDraws<BATCH> dr;
    dr.init(P, seed, (uint32_t)stepR, id);
    constexpr int NA = PROG ? prog_len(PROG) : kMaxActions;
#pragma unroll (PROG ? NA : 1)
    for (int a = 0; a < NA; a++) {
        if ((PROG == 0 && a >= P.n_act) || !alive) break;
        const ActionConst &A = BATCH ? R->act[a] : P.act[a];
        switch (PROG ? prog_act(PROG, a) : A.type) {
        case kGetOld:
            fa = __fsub_rn(fTR, fb);
            break;
        case kFertility:
            if (female) fert = (fa > A.f0) && (fa < A.f1) && (__fsub_rn(fTR, fl) > A.f2);
            else fert = fa > A.f0;
            break;
        case kVerhulst:
        case kVerhulstVarK: {
            uint32_t k = A.window;
            if (cv.tk == 1u) {
                if (female && mated) {
                    if ((uint64_t)dr.get(P, k++) < cv.tb) bflag = true;
                }
            } else if (cv.tk == 2u) {
                if ((uint64_t)dr.get(P, k++) < cv.tb) alive = false;
            }
            if (alive) {
                if ((uint64_t)dr.get(P, k) < cv.td) alive = false;
            }
            if (!alive) cnt_deaths++;
            break;
        }
        case kOldAgeDeath: {
            fa = __fsub_rn(fTR, fb);
            bool die = false;
            if (fa <= A.age_lo) {
                die = false;
            } else if (fa > A.age_hi) {
                die = true;
            } else if (OAD == kOadQueue) {
                queued = true;
            } else if (OAD == kOadGiven) {
                die = oad_die;
            } else {
                const uint32_t u = dr.get(P, A.window);
                const double t = __dmul_rn(__dmul_rn(A.oad_w, (double)u), 2.3283064365386962890625e-10);
                const double thr = __dadd_rn(A.oad_M, __dadd_rn(A.oad_a, t));
                die = (double)fa > thr;
            }
            if (die) { alive = false; cnt_deaths++; }
            break;
        }
        case kATanDeath: {
            // actions/ATanDeath.cpp:57-77: dies if wrandd() < 0.5 + scale *
            // atan(slope * (age - M)) / Q_PI; ages outside the window
            // [age_lo, age_hi] decide without the draw (NaN bounds: none)
            fa = __fsub_rn(fTR, fb);
            bool die;
            if (fa <= A.age_lo) {
                die = false;
            } else if (fa > A.age_hi) {
                die = true;
            } else {
                const double x = __dmul_rn(A.at_slope, __dsub_rn((double)fa, A.at_M));
                const double p = __dadd_rn(0.5, __ddiv_rn(__dmul_rn(A.at_scale, atan(x)), kQPi));
                const uint32_t u = dr.get(P, A.window);
                die = __dmul_rn((double)u, 2.3283064365386962890625e-10) < p;
            }
            if (die) { alive = false; cnt_deaths++; }
            break;
        }
        case kRandomMove: {
            if ((uint64_t)dr.get(P, A.window) < A.pthr) {
                const uint32_t u2 = dr.get(P, A.window + 1);
                const int d = (int)(((uint64_t)(cv.nn + 1u) * (uint64_t)u2) >> 32);
                if (d > 0 && ((cv.vm >> (d - 1)) & 1u)) { dir = d; cnt_moves++; }
            }
            break;
        }
        case kWeightedMove: {
            if ((uint64_t)dr.get(P, A.window) < A.pthr) {
                const uint32_t u2 = dr.get(P, A.window + 1);
                int d;
                if (cv.wf & 1u) {
                    d = (int)(((uint64_t)(cv.nn + 1u) * (uint64_t)u2) >> 32);
                } else {
                    d = 0;
                    const uint64_t *w = wthr + (size_t)cv.c * 6;
                    for (int q = 0; q < (int)cv.nn; q++) d += (w[q] <= (uint64_t)u2) ? 1 : 0;
                }
                // no move into an ice cell (actions/WeightedMove.cpp:91)
                if (d > 0 && ((cv.wv >> (d - 1)) & 1u)) { dir = d; cnt_moves++; }
            }
            break;
        }
        default:
            break;
        }
    }
    const int cls = alive ? (1 + dir) : 0;
    mdir = (uint32_t)dir;
    return (uint8_t)(cls | (bflag ? kOutBirth : 0) | (fert ? kOutFertile : 0) |
                     ((m8 & kMetaGender) ? kOutGender : 0) | (dir > 0 ? kOutMoved : 0));
}

// The actions of a specialised program (Fertility, RandomPair, Verhulst,
// a move, GetOld[, OldAgeDeath]) for one agent, before its mate is known:
// the outcome for both cases where it depends on a mate (a FERTILE female in
// a cell whose Verhulst birth rate is positive: with a mate she draws for a
// birth first and the death draw is the next one).  Bits of the state:
constexpr uint32_t kStDir = 7u;        // move direction (neighbour slot + 1), 0 none
constexpr uint32_t kStFert = 8u;       // FERTILE after Fertility
constexpr uint32_t kStGender = 16u;
constexpr uint32_t kStMateDep = 32u;   // the outcome depends on a mate
constexpr uint32_t kStDeadU = 64u;     // Verhulst kills it (without a mate)
constexpr uint32_t kStDeadM = 128u;    // Verhulst kills it (with a mate)
constexpr uint32_t kStBirthM = 256u;   // gives birth (with a mate)
constexpr int kStOad = 9;              // bits 9-10, OldAgeDeath: 0 survives, 1 dies, 2 inside the window
constexpr uint32_t kStMoveDraw = 2048u; // the move draw passed: the direction is decided later (deferred move)

// With DEFER the move's direction is left out: an agent whose move draw
// passes gets kStMoveDraw and its direction draw in u2out, and move_direction
// decides the direction later, in a dense pass over such agents only (a
// warp's rows rarely all move, so this saves the direction work in most
// lanes).
template <int PROG, bool BATCH, bool DEFER = false>
__device__ __forceinline__ uint32_t agent_state(const StepConst &P, const BatchRun *R, int32_t step, float fT,
                                                int64_t id, uint8_t m8, float fb, float fa, float fl,
                                                const CellView &cv, const uint32_t *wt32, uint32_t wnever,
                                                uint32_t *u2out = nullptr) {
    constexpr int iF = prog_index(PROG, kFertility, kFertility);
    constexpr int iV = prog_index(PROG, kVerhulst, kVerhulstVarK);
    constexpr int iM = prog_index(PROG, kRandomMove, kWeightedMove);
    constexpr int iO = prog_index(PROG, kOldAgeDeath, kOldAgeDeath);
    static_assert(PROG == 0 || (iF >= 0 && iV > iF && iM > iV), "program order: Fertility, Verhulst, move");
    if constexpr (PROG == 0) {
        return 0u;
    } else {
    constexpr bool kWeighted = prog_act(PROG, iM) == kWeightedMove;
    const int32_t stepR = BATCH ? step - R->step0 : step;
    const float fTR = BATCH ? (float)stepR : fT;
    // the Verhulst and move draws lie in the first block of the stream
    constexpr uint32_t kWV = prog_window(PROG, iV), kWM = prog_window(PROG, iM);
    static_assert(kWV + 1u < 4u && kWM + 1u < 4u, "draws outside the first block");
    const Draw4 d = run_block<BATCH>(P, BATCH ? R->seed : P.seed, (uint32_t)stepR, id, kStreamActions);
    const bool female = !(m8 & kMetaGender);
    uint32_t st = female ? 0u : kStGender;
    {   // Fertility::execute (actions/Fertility.cpp:49-73)
        const ActionConst &A = BATCH ? R->act[iF] : P.act[iF];
        const bool fert = female ? (fa > A.f0) && (fa < A.f1) && (__fsub_rn(fTR, fl) > A.f2) : fa > A.f0;
        if (fert) st |= kStFert;
    }
    {   // LinearBirth / LinearDeath ::execute (actions/LinearBirth.cpp:122-166,
        // actions/LinearDeath.cpp:131-150)
        const uint32_t u0 = d.v[kWV], u1 = d.v[kWV + 1u];
        if (cv.tk == 1u) {
            if (female && (m8 & kMetaFertile)) {
                st |= kStMateDep;
                if ((uint64_t)u0 < cv.tb) st |= kStBirthM;
                if ((uint64_t)u1 < cv.td) st |= kStDeadM;
            }
            if ((uint64_t)u0 < cv.td) st |= kStDeadU;
        } else if (cv.tk == 2u) {
            if ((uint64_t)u0 < cv.tb || (uint64_t)u1 < cv.td) st |= kStDeadU;
        } else {
            if ((uint64_t)u0 < cv.td) st |= kStDeadU;
        }
    }
    {   // RandomMove / WeightedMove ::execute (actions/RandomMove.cpp:65-100,
        // actions/WeightedMove.cpp:45-106), for an agent still alive
        const ActionConst &A = BATCH ? R->act[iM] : P.act[iM];
        if (DEFER) {
            if ((uint64_t)d.v[kWM] < A.pthr) st |= kStMoveDraw;
            *u2out = d.v[kWM + 1u];
        } else if ((uint64_t)d.v[kWM] < A.pthr) {
            const uint32_t u2 = d.v[kWM + 1u];
            int d;
            if (!kWeighted || (cv.wf & 1u)) {
                d = (int)(((uint64_t)(cv.nn + 1u) * (uint64_t)u2) >> 32);
            } else {
                // the number of slots whose threshold (a running maximum, 2^32
                // past the neighbours) is <= u2: in 32 bits every slot counts
                // correctly except a 2^32 threshold against u2 = 0xffffffff,
                // which the never mask takes back out
                const uint4 wa = *reinterpret_cast<const uint4 *>(wt32);
                const uint2 wb = *reinterpret_cast<const uint2 *>(wt32 + 4);
                d = (wa.x <= u2 ? 1 : 0) + (wa.y <= u2 ? 1 : 0) + (wa.z <= u2 ? 1 : 0) + (wa.w <= u2 ? 1 : 0) +
                    (wb.x <= u2 ? 1 : 0) + (wb.y <= u2 ? 1 : 0);
                if (u2 == 0xffffffffu) d -= __popc(wnever);
            }
            // WeightedMove registers no move into an ice cell (actions/WeightedMove.cpp:91)
            if (d > 0 && (((kWeighted ? cv.wv : cv.vm) >> (d - 1)) & 1u)) st |= (uint32_t)d;
        }
    }
    if (iO >= 0) {   // OldAgeDeath::execute (actions/OldAgeDeath.cpp:48-67): the window test
        const ActionConst &A = BATCH ? R->act[iO > 0 ? iO : 0] : P.act[iO > 0 ? iO : 0];
        const float fa2 = __fsub_rn(fTR, fb);
        const uint32_t o = (fa2 <= A.age_lo) ? 0u : ((fa2 > A.age_hi) ? 1u : 2u);
        st |= o << kStOad;
    }
    return st;
    }
}

// The direction of an agent whose move draw passed (RandomMove::execute,
// actions/RandomMove.cpp:65-100; WeightedMove::execute,
// actions/WeightedMove.cpp:45-106): neighbour slot + 1, 0 when it stays or
// the slot holds no cell (for WeightedMove also when the cell is ice,
// actions/WeightedMove.cpp:91)
template <bool kWeighted>
__device__ __forceinline__ uint32_t move_direction(const CellView &cv, const uint32_t *wt32, uint32_t wnever,
                                                   uint32_t u2) {
    int d;
    if (!kWeighted || (cv.wf & 1u)) {
        d = (int)(((uint64_t)(cv.nn + 1u) * (uint64_t)u2) >> 32);
    } else {
        // see agent_state: slots whose threshold is <= u2, in 32 bits with
        // the unreachable thresholds taken back out for u2 = 0xffffffff
        const uint4 wa = *reinterpret_cast<const uint4 *>(wt32);
        const uint2 wb = *reinterpret_cast<const uint2 *>(wt32 + 4);
        d = (wa.x <= u2 ? 1 : 0) + (wa.y <= u2 ? 1 : 0) + (wa.z <= u2 ? 1 : 0) + (wa.w <= u2 ? 1 : 0) +
            (wb.x <= u2 ? 1 : 0) + (wb.y <= u2 ? 1 : 0);
        if (u2 == 0xffffffffu) d -= __popc(wnever);
    }
    return (d > 0 && (((kWeighted ? cv.wv : cv.vm) >> (d - 1)) & 1u)) ? (uint32_t)d : 0u;
}

template <int PROG, bool BATCH, bool BIG>
__global__ void __launch_bounds__(Tile<BIG>::kThreads, BIG ? 1 : 4)
k_actions(const StepConst P, const BatchBuffers BB, RunState *__restrict__ rs,
          const uint32_t *__restrict__ nonempty, const uint32_t *__restrict__ ne_start,
          const uint32_t *__restrict__ tile_first,
          const int64_t *__restrict__ id, const float *__restrict__ birth,
          const float *__restrict__ age, const float *__restrict__ lastb,
          const uint8_t *__restrict__ meta,
          const ulonglong2 *__restrict__ vthr, const uint64_t *__restrict__ wthr,
          const uint32_t *__restrict__ necm,
          uint32_t *__restrict__ outc, int32_t *__restrict__ father, uint16_t *__restrict__ brank,
          uint32_t *__restrict__ clsc) {
    constexpr int TT = Tile<BIG>::kThreads;
    constexpr int TM = Tile<BIG>::kMax;
    extern __shared__ __align__(16) unsigned char qhg_smem[];
    ActionsSmemT<TM, TT, BATCH> &S = *reinterpret_cast<ActionsSmemT<TM, TT, BATCH> *>(qhg_smem);
    if (rs->error != 0u) return;   // an earlier kernel failed: keep the state
    if (rs->form != (BIG ? kFormBig : kFormTile)) return;   // another form runs this step
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int32_t step = rs->step;
    const float fT = (float)step;
    // the table's ages: derived from birth times once a step of a single run has run
    const bool derived = !BATCH && rs->age_derived != 0u;
    const float fTprev = (float)(step - 1);
    const uint32_t N = rs->n_agents;
    const uint32_t ntiles = (N + kTileAgents - 1) / kTileAgents;
    uint32_t cnt_births = 0, cnt_deaths = 0, cnt_moves = 0;
    constexpr int RA = TM / TT;
    constexpr bool kDeferOad = prog_defers_oad(PROG);

    // tiles are dealt out statically.  The bounds of the CTA's next tile
    // (first non-empty cell, first row) are loaded one tile ahead, so that a
    // tile's agent fields and cell data are requested together at its start
    uint32_t nr0 = 0, nr1 = 0, na0 = 0, na1 = 0;
    if (blockIdx.x < ntiles) {
        nr0 = tile_first[blockIdx.x];
        nr1 = tile_first[blockIdx.x + 1];
        na0 = ne_start[nr0];
        na1 = ne_start[nr1];
    }
    for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const uint32_t r0 = nr0;
        const int nc = (int)(nr1 - r0);
        const uint32_t a0 = na0;
        const int na = (int)(na1 - na0);
        const uint32_t tn = t + gridDim.x;
        if (tn < ntiles) {
            nr0 = tile_first[tn];
            nr1 = tile_first[tn + 1];
        }
        if (nc == 0 || na > TM || nc > kTileCells) {
            if (nc != 0 && tid == 0) set_error(rs, kErrCellTooLarge, r0);
            if (tn < ntiles) {
                na0 = ne_start[nr0];
                na1 = ne_start[nr1];
            }
            continue;
        }
        int64_t pid[RA];
        uint8_t pm[RA];
        float pb[RA], pa[RA], pl[RA];
#pragma unroll
        for (int j = 0; j < RA; j++) {
            const int i = tid + j * TT;
            if (i < na) {
                pid[j] = id[a0 + i];
                pm[j] = meta[a0 + i];
                pb[j] = birth[a0 + i];
                pa[j] = P.reads_age ? (derived ? __fsub_rn(fTprev, pb[j]) : age[a0 + i]) : 0.0f;
                pl[j] = lastb[a0 + i];
            }
        }
        __syncthreads();   // the previous tile is done with the shared arrays
        // ---- cells: ids, rows, Verhulst thresholds (LinearBirth / LinearDeath
        // ::initialize, actions/LinearBirth.cpp:90-112, actions/LinearDeath.cpp:92-122)
        // and move words, both stored by position in the non-empty list
        for (int lc = tid; lc < nc; lc += TT) {
            const uint32_t r = r0 + (uint32_t)lc;
            const uint32_t c = nonempty[r];
            const uint32_t cs = ne_start[r] - a0;
            uint32_t cm = 0u;
            ulonglong2 v = make_ulonglong2(0ull, 0ull);
            if (P.has_move) cm = necm[r];
            if (P.n_verhulst > 0) v = vthr[r];   // computed by the previous step's cell scan
            S.cid[lc] = (int32_t)c;
            S.cstart[lc] = cs;
            if (lc == nc - 1) S.cstart[nc] = (uint32_t)na;
            if (BATCH) {
                S.crun[lc] = BB.crun[c];
                S.dm[lc] = 0u;
            }
            S.nfm[lc] = 0u;
            S.cls[lc][0] = S.cls[lc][1] = S.cls[lc][2] = S.cls[lc][3] = 0u;
            // the neighbour row of the cell as a count and a mask of valid slots,
            // so that moving agents read no neighbour data from memory
            S.nn[lc] = (uint8_t)(cm & 7u);
            S.vm[lc] = (uint8_t)((cm >> 8) & 63u);
            S.wv[lc] = (uint8_t)((cm >> 24) & 63u);
            S.wf[lc] = (uint8_t)((cm >> 16) & 1u);
            S.tk[lc] = (uint8_t)(v.x >> 62);
            S.tb[lc] = v.x & ((1ull << 62) - 1ull);
            S.td[lc] = v.y;
            if (P.has_wmove) asm volatile("prefetch.global.L1 [%0];" ::"l"(wthr + (size_t)c * 6));
        }
#pragma unroll
        for (int j = 0; j < RA; j++) {
            const int i = tid + j * TT;
            if (i < na) S.mate[i] = -1;
        }
        if (tid == 0) { S.npick = 0u; S.noad = 0u; S.nfert = 0u; S.idhi = 0u; }
        __syncthreads();
        // local cell of each row: binary search of the cells' first rows (the
        // searches of a thread's rows run side by side)
        {
            int lo[RA];
#pragma unroll
            for (int j = 0; j < RA; j++) lo[j] = 0;
            for (int s = 1 << (31 - __clz(nc)); s > 0; s >>= 1) {
#pragma unroll
                for (int j = 0; j < RA; j++) {
                    const int m = lo[j] + s;
                    if (m < nc && (int)S.cstart[m] <= tid + j * TT) lo[j] = m;
                }
            }
#pragma unroll
            for (int j = 0; j < RA; j++) {
                const int i = tid + j * TT;
                if (i < na) S.cell[i] = (uint16_t)lo[j];
            }
        }
        if (BATCH) {
            // agents of a run that leaves the batch take no part in pairing
#pragma unroll
            for (int j = 0; j < RA; j++) {
                const int i = tid + j * TT;
                if (i < na && !BB.runs[S.crun[S.cell[i]]].active) pm[j] &= (uint8_t)~kMetaFertile;
            }
        }
        // ---- RandomPair::findMates (actions/RandomPair.cpp:146-270), members in
        // ID order, each pick drawn from the pairing stream of the picking member
        if (P.has_pair) {
            // unsorted FERTILE lists: females from the cell's first row up, males
            // from its last row down (with their IDs beside them)
#pragma unroll
            for (int j = 0; j < RA; j++) {
                const int i = tid + j * TT;
                if (__all_sync(FULL_MASK, i >= na)) break;
                const uint8_t m = (i < na) ? pm[j] : (uint8_t)0;
                const bool fert = (m & kMetaFertile) != 0;
                const bool male = (m & kMetaGender) != 0;
                const int lc = fert ? S.cell[i] : 0;
                const uint32_t q0 = warp_agg_add(fert, ((uint32_t)lc << 1) | (male ? 1u : 0u), &S.nfm[lc],
                                                 male ? 0x10000u : 1u);
                const uint32_t q = male ? (q0 >> 16) : (q0 & 0xffffu);
                // the tile's FERTILE agents also go to a dense list (their list
                // positions), so that the rank loop below runs on full warps
                const uint32_t fb = __ballot_sync(FULL_MASK, fert);
                uint32_t fbase = 0;
                if (lane == 0 && fb) fbase = atomicAdd(&S.nfert, (uint32_t)__popc(fb));
                fbase = __shfl_sync(FULL_MASK, fbase, 0);
                if (fert) {
                    const uint32_t pos = male ? (S.cstart[lc + 1] - 1u - q) : (S.cstart[lc] + q);
                    S.pick[pos] = (uint16_t)i;
                    S.fid[pos] = pid[j];
                    S.oadq[fbase + __popc(fb & lanemask_lt())] = (uint16_t)pos;
                }
                // high words of the IDs: the ranks compare 32-bit keys while all are zero
                const uint32_t hi = __reduce_or_sync(FULL_MASK, fert ? (uint32_t)((uint64_t)pid[j] >> 32) : 0u);
                if (lane == 0 && hi) atomicOr(&S.idhi, hi);
            }
            __syncthreads();
            // rank by ID within the own sex's list (IDs are unique), over the
            // dense list of FERTILE agents; each agent goes to its place in its
            // cell's ID-ordered lists (females, then males), and the members of
            // the smaller side (the picking side) to the dense list of pickers
            const uint32_t nfe = S.nfert;
            const bool k32 = S.idhi == 0u;
            const uint32_t *f32 = reinterpret_cast<const uint32_t *>(S.fid);
            for (uint32_t qb = 0; qb < nfe; qb += TT) {
                const uint32_t q = qb + (uint32_t)tid;
                bool picker = false;
                int pos = 0;
                if (q < nfe) {
                    pos = S.oadq[q];
                    const int i = S.pick[pos];
                    const int lc = S.cell[i];
                    const int cs = (int)S.cstart[lc], ce = (int)S.cstart[lc + 1];
                    const uint32_t w = S.nfm[lc];
                    const int nF = (int)(w & 0xffffu), nM = (int)(w >> 16);
                    const bool male = pos >= cs + nF;
                    const int b = male ? ce - nM : cs;
                    const int e = male ? ce : cs + nF;
                    int r = 0;
                    if (k32) {
                        const uint32_t x = f32[2 * pos];
                        int k = b;
                        for (; k + 4 <= e; k += 4) {
                            r += (f32[2 * k] < x ? 1 : 0) + (f32[2 * k + 2] < x ? 1 : 0) +
                                 (f32[2 * k + 4] < x ? 1 : 0) + (f32[2 * k + 6] < x ? 1 : 0);
                        }
                        for (; k < e; k++) r += (f32[2 * k] < x) ? 1 : 0;
                    } else {
                        const int64_t x = S.fid[pos];
                        for (int k = b; k < e; k++) r += (S.fid[k] < x) ? 1 : 0;
                    }
                    S.frank[i] = (uint16_t)r;
                    S.list[cs + (male ? nF : 0) + r] = (uint16_t)i;
                    picker = nF > 0 && nM > 0 && (male == (nM < nF));
                }
                const uint32_t pk = __ballot_sync(FULL_MASK, picker);
                uint32_t pbase = 0;
                if (lane == 0 && pk) pbase = atomicAdd(&S.npick, (uint32_t)__popc(pk));
                pbase = __shfl_sync(FULL_MASK, pbase, 0);
                if (picker) S.pkpos[pbase + __popc(pk & lanemask_lt())] = (uint16_t)pos;
            }
            __syncthreads();
            // pick j takes the pick[j]-th still unpaired member of the larger
            // side, pick[j] = (int)wrandr(0, nL - j)
            const uint32_t npk = S.npick;
            for (uint32_t q = tid; q < npk; q += TT) {
                const int pos = S.pkpos[q];
                const int i = S.pick[pos];
                const int lc = S.cell[i];
                const uint32_t w = S.nfm[lc];
                const uint32_t nF = w & 0xffffu, nM = w >> 16;
                const uint32_t nL = (nF <= nM) ? nM : nF;
                const uint32_t j = S.frank[i];
                uint64_t sd = P.seed;
                int32_t st = step;
                if (BATCH) {
                    const BatchRun &R = BB.runs[S.crun[lc]];
                    sd = R.seed;
                    st = step - R.step0;
                }
                const uint32_t u = run_block<BATCH>(P, sd, (uint32_t)st, S.fid[pos], kStreamPair).v[0];
                S.oadq[S.cstart[lc] + j] = (uint16_t)(((uint64_t)(nL - j) * (uint64_t)u) >> 32);
            }
            __syncthreads();
            // the member taken by pick j, decoded on its own: start from pick[j]
            // and for i = j-1 down to 0 step over the member pick i took when it
            // lies at or below
            for (uint32_t q = tid; q < npk; q += TT) {
                const int i = S.pick[S.pkpos[q]];
                const int lc = S.cell[i];
                const uint32_t w = S.nfm[lc];
                const uint32_t nF = w & 0xffffu, nM = w >> 16;
                const bool femSmall = nF <= nM;
                const int cs = (int)S.cstart[lc];
                const int j = S.frank[i];
                uint32_t p = S.oadq[cs + j];
                for (int k = j - 1; k >= 0; k--) p += (p >= S.oadq[cs + k]) ? 1u : 0u;
                const uint32_t nL = femSmall ? nM : nF;
                if (p >= nL) {   // cannot happen: every pick finds a free member
                    set_error(rs, kErrInternal, 1u);
                } else {
                    const int partner = S.list[cs + (femSmall ? (int)nF : 0) + (int)p];
                    S.mate[i] = (int16_t)partner;
                    S.mate[partner] = (int16_t)i;
                }
            }
            __syncthreads();
        }
        // the next tile's first row and end, requested while this tile works
        if (tn < ntiles) {
            na0 = ne_start[nr0];
            na1 = ne_start[nr1];
        }
        // ---- every action on every agent (SPopulation::doActions), then the
        // outcome word with the agent's rank in its cell's class; agents
        // inside the OldAgeDeath window wait for the dense pass below
        uint32_t mothers = 0u;   // bit j: row tid + j*TT gives birth
#pragma unroll
        for (int j = 0; j < RA; j++) {
            const int i = tid + j * TT;
            if (__all_sync(FULL_MASK, i >= na)) break;
            const bool in_tile = i < na;
            uint8_t oc = 0;
            uint32_t mdir = 0u;
            bool queued = false;
            float fa = 0.0f;
            int lc = 0;
            if (in_tile) {
                const uint32_t row = a0 + (uint32_t)i;
                lc = S.cell[i];
                const int c = S.cid[lc];
                const uint8_t m8 = pm[j];
                const BatchRun *R = BATCH ? BB.runs + S.crun[lc] : nullptr;
                if (BATCH && !R->active) {   // the run leaves the batch: drop its agents
                    oc = kOutDropped;
                } else {
                    CellView cv;
                    cv.tk = S.tk[lc];
                    cv.tb = S.tb[lc];
                    cv.td = S.td[lc];
                    cv.nn = S.nn[lc];
                    cv.vm = S.vm[lc];
                    cv.wv = S.wv[lc];
                    cv.wf = S.wf[lc];
                    cv.c = (uint32_t)c;
                    const int mate = S.mate[i];
                    oc = agent_outcome<PROG, BATCH, kDeferOad ? kOadQueue : kOadDraw>(
                        P, R, step, fT, pid[j], m8, pb[j], pa[j], pl[j], mate >= 0, cv, wthr, false, fa, queued,
                        cnt_deaths, cnt_moves, mdir);
                    if (oc & kOutBirth) {
                        father[row] = (int32_t)(a0 + (uint32_t)mate);
                        cnt_births++;
                        mothers |= 1u << j;
                    }
                }
                S.oc[i] = oc;
            }
            if (kDeferOad) {
                const uint32_t qm = __ballot_sync(FULL_MASK, queued);
                if (qm) {
                    uint32_t qbase = 0;
                    if (lane == 0) qbase = atomicAdd(&S.noad, (uint32_t)__popc(qm));
                    qbase = __shfl_sync(FULL_MASK, qbase, 0);
                    if (queued) {
                        const uint32_t q = qbase + __popc(qm & lanemask_lt());
                        S.oadq[q] = (uint16_t)i;
                        S.fid[q] = pid[j];
                        S.ofa[q] = fa;
                    }
                }
            }
            // outcome word: outcome byte | local cell << 8 | rank in the cell's
            // class << 17; for the dead, the direction of a move they registered
            const int cls = oc & 7;
            const uint32_t rank = class_rank(in_tile && !queued && cls > 0, lc, cls, S.cls);
            if (in_tile && !queued)
                outc[a0 + (uint32_t)i] = (uint32_t)oc | ((uint32_t)lc << 8) | ((cls > 0 ? rank : mdir) << 17);
            // mothers: a list per cell of their ID ranks (births are rare: most
            // warps have none and skip the aggregation)
            const bool mother = (mothers >> j) & 1u;
            if (__any_sync(FULL_MASK, mother)) {
                const uint32_t mq = warp_agg_add(mother, ((uint32_t)lc << 3) | 7u, &S.cls[lc][3], 1u << 16) >> 16;
                if (mother) S.pick[S.cstart[lc] + mq] = S.frank[i];
            }
            if (BATCH) {
                const bool died = in_tile && !queued && cls == 0 && !(oc & kOutDropped);
                const bool moved = in_tile && !queued && (oc & kOutMoved);
                if (__any_sync(FULL_MASK, died)) warp_agg_add(died, (uint32_t)lc, &S.dm[lc], 1u);
                if (__any_sync(FULL_MASK, moved)) warp_agg_add(moved, (uint32_t)lc, &S.dm[lc], 1u << 16);
            }
        }
        if (kDeferOad) {
            // OldAgeDeath::execute (actions/OldAgeDeath.cpp:57-60) for the agents
            // inside the death window: age > M + wrandr(1 - U*M, 1 + U*M)
            __syncthreads();
            const uint32_t nq = S.noad;
            constexpr int kOad = prog_len(PROG) - 1;
            for (uint32_t qb = 0; qb < nq; qb += TT) {
                const uint32_t q = qb + (uint32_t)tid;
                const bool valid = q < nq;
                int i = 0, lc = 0;
                uint8_t oc = 0;
                uint32_t mdir = 0u;
                if (valid) {
                    i = S.oadq[q];
                    lc = S.cell[i];
                    oc = S.oc[i];
                    const BatchRun *R = BATCH ? BB.runs + S.crun[lc] : nullptr;
                    const ActionConst &A = BATCH ? R->act[kOad] : P.act[kOad];
                    const int32_t stepR = BATCH ? step - R->step0 : step;
                    const uint32_t w = A.window;
                    const uint32_t u = pick4(run_block<BATCH>(P, BATCH ? R->seed : P.seed, (uint32_t)stepR, S.fid[q],
                                                        kStreamActions + (w >> 2)), w & 3u);
                    const double th = __dmul_rn(__dmul_rn(A.oad_w, (double)u), 2.3283064365386962890625e-10);
                    const double thr = __dadd_rn(A.oad_M, __dadd_rn(A.oad_a, th));
                    if ((double)S.ofa[q] > thr) {
                        const uint32_t c0 = oc & 7u;   // alive until now: 1 + its move direction
                        mdir = c0 >= 2u ? c0 - 1u : 0u;
                        oc = (uint8_t)(oc & ~7u);
                        cnt_deaths++;
                    }
                }
                const int cls = oc & 7;
                const uint32_t rank = class_rank(valid && cls > 0, lc, cls, S.cls);
                if (valid) outc[a0 + (uint32_t)i] = (uint32_t)oc | ((uint32_t)lc << 8) | ((cls > 0 ? rank : mdir) << 17);
                if (BATCH) {
                    const bool died = valid && cls == 0;
                    const bool moved = valid && (oc & kOutMoved);
                    if (__any_sync(FULL_MASK, died)) warp_agg_add(died, (uint32_t)lc, &S.dm[lc], 1u);
                    if (__any_sync(FULL_MASK, moved)) warp_agg_add(moved, (uint32_t)lc, &S.dm[lc], 1u << 16);
                }
            }
        }
        __syncthreads();
        // ---- per cell: the class counts; per mother: her birth rank, the
        // number of her cell's mothers with a smaller ID (births are numbered
        // in (cell, mother ID) order)
        for (int lc = tid; lc < nc; lc += TT) {
            const uint32_t c = (uint32_t)S.cid[lc];
            uint4 *dst = reinterpret_cast<uint4 *>(clsc + (size_t)c * kCls);
            const uint32_t w0 = S.cls[lc][0], w1 = S.cls[lc][1], w2 = S.cls[lc][2], w3 = S.cls[lc][3];
            dst[0] = make_uint4(w0 & 0xffffu, w0 >> 16, w1 & 0xffffu, w1 >> 16);
            dst[1] = make_uint4(w2 & 0xffffu, w2 >> 16, w3 & 0xffffu, w3 >> 16);
            if (BATCH) BB.cstat[c] = S.dm[lc];   // deaths | registered moves << 16
        }
#pragma unroll
        for (int j = 0; j < RA; j++) {
            if (!((mothers >> j) & 1u)) continue;
            const int i = tid + j * TT;
            const int lc = S.cell[i];
            const int cs = (int)S.cstart[lc];
            const int nmo = (int)(S.cls[lc][3] >> 16);
            const uint32_t fr = S.frank[i];
            uint32_t r = 0;
            for (int k = 0; k < nmo; k++) r += (S.pick[cs + k] < fr) ? 1u : 0u;
            brank[a0 + (uint32_t)i] = (uint16_t)r;
        }
    }
    // statistics of the step (batches: per run, by the cell scan)
    if (BATCH) return;
    const uint32_t tb_ = block_sum(cnt_births, S.red);
    const uint32_t td_ = block_sum(cnt_deaths, S.red);
    const uint32_t tm_ = block_sum(cnt_moves, S.red);
    if (tid == 0 && (tb_ | td_ | tm_)) {
        unsigned long long *st = rs->stats[(uint32_t)step % kStatsRing];
        atomicAdd(&st[1], (unsigned long long)tb_);
        atomicAdd(&st[2], (unsigned long long)td_);
        atomicAdd(&st[3], (unsigned long long)tm_);
    }
}

// --------------------------------------------------------------- cell scan
struct ScanVal {
    uint32_t n, b, ne;
};

__device__ __forceinline__ ScanVal sv_add(ScanVal x, ScanVal y) {
    ScanVal r;
    r.n = x.n + y.n; r.b = x.b + y.b; r.ne = x.ne + y.ne;
    return r;
}

__device__ __forceinline__ ScanVal sv_shfl_up(ScanVal v, int o) {
    ScanVal r;
    r.n = __shfl_up_sync(FULL_MASK, v.n, o);
    r.b = __shfl_up_sync(FULL_MASK, v.b, o);
    r.ne = __shfl_up_sync(FULL_MASK, v.ne, o);
    return r;
}

__device__ __forceinline__ ScanVal sv_shfl_down(ScanVal v, int o) {
    ScanVal r;
    r.n = __shfl_down_sync(FULL_MASK, v.n, o);
    r.b = __shfl_down_sync(FULL_MASK, v.b, o);
    r.ne = __shfl_down_sync(FULL_MASK, v.ne, o);
    return r;
}

// Look-back status words: (epoch << 2) | 1 aggregate ready, | 2 inclusive
// prefix ready.  The epoch is the step number, so words of earlier steps read
// as not ready; the host clears them whenever the step counter is reset.
// Per-run sums of a batch step over the cells a warp holds: one atomic per
// run and value; lanes with r == kNoRun add nothing.
__device__ __forceinline__ void batch_run_stats(uint32_t *rstat, uint32_t slot, uint32_t r, uint32_t n,
                                                uint32_t b, uint32_t d, uint32_t m) {
    const int lane = threadIdx.x & 31;
    uint32_t todo = __ballot_sync(FULL_MASK, r != kNoRun);
    while (todo) {
        const int leader = __ffs(todo) - 1;
        const uint32_t rr = __shfl_sync(FULL_MASK, r, leader);
        const bool mine = (r == rr);
        const uint32_t sn = __reduce_add_sync(FULL_MASK, mine ? n : 0u);
        const uint32_t sb = __reduce_add_sync(FULL_MASK, mine ? b : 0u);
        const uint32_t sd = __reduce_add_sync(FULL_MASK, mine ? d : 0u);
        const uint32_t sm = __reduce_add_sync(FULL_MASK, mine ? m : 0u);
        if (lane == leader) {
            uint32_t *q = rstat + ((size_t)rr * kBatchRing + slot) * 4;
            if (sn) atomicAdd(q + 0, sn);
            if (sb) atomicAdd(q + 1, sb);
            if (sd) atomicAdd(q + 2, sd);
            if (sm) atomicAdd(q + 3, sm);
        }
        todo &= ~__ballot_sync(FULL_MASK, mine);
    }
}

template <bool BATCH, int ITEMS>
__global__ void __launch_bounds__(kScanThreads)
k_cell_scan(const StepConst P, const BatchBuffers BB, RunState *__restrict__ rs,
            const int32_t *__restrict__ nbr, const uint8_t *__restrict__ nnbr,
            const uint32_t *__restrict__ rev, const uint32_t *__restrict__ clsc,
            const double *__restrict__ Kc, ulonglong2 *__restrict__ vthr,
            const uint32_t *__restrict__ cmove, uint32_t *__restrict__ necm,
            uint32_t *__restrict__ sbase, uint32_t *__restrict__ bbase,
            uint32_t *__restrict__ bidbase, uint32_t *__restrict__ obase,
            uint32_t *__restrict__ new_nonempty, uint32_t *__restrict__ new_ne_start,
            uint32_t *__restrict__ new_tile_first,
            uint32_t *__restrict__ tile_flag, uint4 *__restrict__ tile_agg, uint4 *__restrict__ tile_incl) {
    __shared__ uint32_t s_tile;
    __shared__ ScanVal s_warp[kScanThreads / 32];
    __shared__ ScanVal s_prefix;
    if (rs->error != 0u) return;
    const int C = P.num_cells;
    constexpr int kTile = kScanThreads * ITEMS;
    const uint32_t ntiles = (uint32_t)((C + kTile - 1) / kTile);
    const uint32_t epoch = ((uint32_t)rs->step + 1u) & 0x3fffffffu;
    if (threadIdx.x == 0) {
        const uint32_t t = atomicAdd(&rs->scan_tiles_started, 1u);
        if (t == ntiles - 1) rs->scan_tiles_started = 0u;
        s_tile = t;
    }
    __syncthreads();
    const uint32_t tile = s_tile;
    // a tile counter that did not start at zero hands out numbers past the
    // last tile: never index past the status arrays (the tile left out makes
    // its successor's bounded wait fail and report the step)
    if (tile >= ntiles) return;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int base = (int)tile * kTile + threadIdx.x * ITEMS;
    // a test of the bounded waits withholds this tile's status once: its
    // successor's look-back runs out, the step fails with kErrTimeout
    const bool withhold = (rs->stall_tile == tile + 1u);
    if (withhold && threadIdx.x == 0) rs->stall_tile = 0u;

    uint32_t nnew[ITEMS], stay[ITEMS], bth[ITEMS];
    uint32_t crn[ITEMS];
    uint32_t rsum_n = 0u, rsum_b = 0u, rsum_d = 0u, rsum_m = 0u, rcur = kNoRun;
    ScanVal loc = {0u, 0u, 0u};
#pragma unroll
    for (int j = 0; j < ITEMS; j++) {
        const int d = base + j;
        nnew[j] = stay[j] = bth[j] = 0u;
        crn[j] = kNoRun;
        if (d < C) {
            // class counts of empty cells are zero (cleared by the scatter)
            const uint32_t st = clsc[(size_t)d * kCls + 0];
            const uint32_t bt = clsc[(size_t)d * kCls + 7];
            const int nn = nnbr[d];
            const uint32_t rv = rev[d];
            uint32_t mvin = 0;
            for (int q = 0; q < nn; q++) {
                const int sn = nbr[d * 6 + q];
                if (sn >= 0) mvin += clsc[(size_t)sn * kCls + 1 + ((rv >> (3 * q)) & 7u)];
            }
            stay[j] = st;
            bth[j] = bt;
            nnew[j] = st + mvin + bt;
            if (BATCH) {
                const uint32_t r = BB.crun[d];
                crn[j] = r;
                nnew[j] += BB.inj[d];
                if (r != kNoRun) {
                    // cells of a thread are consecutive: one run or two
                    if (r != rcur) {
                        if (rcur != kNoRun) {
                            uint32_t *q = BB.rstat + ((size_t)rcur * kBatchRing + (uint32_t)rs->step % kBatchRing) * 4;
                            if (rsum_n) atomicAdd(q + 0, rsum_n);
                            if (rsum_b) atomicAdd(q + 1, rsum_b);
                            if (rsum_d) atomicAdd(q + 2, rsum_d);
                            if (rsum_m) atomicAdd(q + 3, rsum_m);
                        }
                        rcur = r;
                        rsum_n = rsum_b = rsum_d = rsum_m = 0u;
                    }
                    const uint32_t cs = BB.cstat[d];
                    if (cs) BB.cstat[d] = 0u;   // consumed
                    rsum_n += nnew[j];
                    rsum_b += bt;
                    rsum_d += cs & 0xffffu;
                    rsum_m += cs >> 16;
                }
            }
            loc.n += nnew[j];
            loc.b += bt;
            loc.ne += (nnew[j] > 0u) ? 1u : 0u;
        }
    }
    if (BATCH) batch_run_stats(BB.rstat, (uint32_t)rs->step % kBatchRing, rcur, rsum_n, rsum_b, rsum_d, rsum_m);
    // block scan of the per-thread totals
    ScanVal inc = loc;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const ScanVal y = sv_shfl_up(inc, o);
        if (lane >= o) inc = sv_add(inc, y);
    }
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const ScanVal wv = (lane < kScanThreads / 32) ? s_warp[lane] : ScanVal{0u, 0u, 0u};
        ScanVal wi = wv;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const ScanVal y = sv_shfl_up(wi, o);
            if (lane >= o) wi = sv_add(wi, y);
        }
        if (lane < kScanThreads / 32) s_warp[lane] = ScanVal{wi.n - wv.n, wi.b - wv.b, wi.ne - wv.ne};
        const ScanVal total = {__shfl_sync(FULL_MASK, wi.n, kScanThreads / 32 - 1),
                               __shfl_sync(FULL_MASK, wi.b, kScanThreads / 32 - 1),
                               __shfl_sync(FULL_MASK, wi.ne, kScanThreads / 32 - 1)};
        ScanVal excl = {0u, 0u, 0u};
        if (tile == 0) {
            if (lane == 0) {
                tile_incl[tile] = make_uint4(total.n, total.b, total.ne, 0u);
                __threadfence();
                if (!withhold) atomicExch(&tile_flag[tile], (epoch << 2) | 2u);
            }
        } else {
            if (lane == 0) {
                tile_agg[tile] = make_uint4(total.n, total.b, total.ne, 0u);
                __threadfence();
                if (!withhold) atomicExch(&tile_flag[tile], (epoch << 2) | 1u);
            }
            // warp-wide look-back over windows of 32 predecessors
            int wbase = (int)tile - 1;
            uint32_t spins = 0;
            const uint64_t t_start = globaltimer_ns();
            while (true) {
                const int tt = wbase - lane;
                uint32_t f = (epoch << 2) | 2u;   // before tile 0: an inclusive prefix of zero
                if (tt >= 0) f = atomicAdd(&tile_flag[tt], 0u);
                const bool ready = (tt < 0) || (((f >> 2) == epoch) && ((f & 3u) != 0u));
                if (__all_sync(FULL_MASK, ready)) {
                    __threadfence();
                    const bool incl = (tt < 0) || ((f & 3u) == 2u);
                    ScanVal v = {0u, 0u, 0u};
                    if (tt >= 0) {
                        const uint4 q = incl ? __ldcg(&tile_incl[tt]) : __ldcg(&tile_agg[tt]);
                        v = ScanVal{q.x, q.y, q.z};
                    }
                    const uint32_t im = __ballot_sync(FULL_MASK, incl);
                    // lanes up to the first inclusive one (nearest predecessor) contribute
                    const int stop = im ? (__ffs(im) - 1) : 31;
                    if (lane > stop) v = ScanVal{0u, 0u, 0u};
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) v = sv_add(v, sv_shfl_down(v, o));
                    excl = sv_add(excl, ScanVal{__shfl_sync(FULL_MASK, v.n, 0), __shfl_sync(FULL_MASK, v.b, 0),
                                                __shfl_sync(FULL_MASK, v.ne, 0)});
                    if (im) break;
                    wbase -= 32;
                } else if (++spins > kSpinLimit || globaltimer_ns() - t_start > kWaitLimitNs) {
                    // a predecessor never published: give up, report, return
                    if (lane == 0) set_error(rs, kErrTimeout, tile);
                    break;
                }
            }
            if (lane == 0) {
                tile_incl[tile] = make_uint4(excl.n + total.n, excl.b + total.b, excl.ne + total.ne, 0u);
                __threadfence();
                if (!withhold) atomicExch(&tile_flag[tile], (epoch << 2) | 2u);
            }
        }
        if (lane == 0) {
            s_prefix = excl;
            if (tile == ntiles - 1) {
                const uint32_t tn = excl.n + total.n;
                const uint32_t tne = excl.ne + total.ne;
                rs->new_n_agents = tn;
                rs->new_n_nonempty = tne;
                rs->births = excl.b + total.b;
                new_ne_start[tne] = tn;
                if (tn <= P.capacity) new_tile_first[(tn + kTileAgents - 1) / kTileAgents] = tne;
                if (tn > P.capacity) set_error(rs, kErrCapacity, tn);
            }
        }
    }
    __syncthreads();
    uint32_t cmax = 0u;   // largest cell of this thread in the next table
    ScanVal pre = sv_add(s_prefix, s_warp[warp]);
    {
        const ScanVal y = sv_shfl_up(inc, 1);
        if (lane >= 1) pre = sv_add(pre, y);
    }
#pragma unroll
    for (int j = 0; j < ITEMS; j++) {
        const int d = base + j;
        if (d < C) {
            sbase[d] = pre.n;
            bidbase[d] = pre.b;
            uint32_t run = pre.n + stay[j];
            const int nn = nnbr[d];
            const uint32_t rv = rev[d];
            for (int q = 0; q < nn; q++) {
                const int sn = nbr[d * 6 + q];
                if (sn >= 0) {
                    const uint32_t k = (rv >> (3 * q)) & 7u;
                    const uint32_t m = clsc[(size_t)sn * kCls + 1 + k];
                    if (m) obase[(size_t)sn * 6 + k] = run;
                    run += m;
                }
            }
            bbase[d] = run;
            if (BATCH && BB.inj[d] > 0u) BB.ibase[d] = run + bth[j];   // admitted agents follow the newborns
            if (nnew[j] > 0u) {
                new_nonempty[pre.ne] = (uint32_t)d;
                new_ne_start[pre.ne] = pre.n;
                // the next step's Verhulst thresholds and move word of the cell, by
                // its position in the next table's non-empty list
                if (P.n_verhulst > 0) {
                    if (!BATCH) {
                        vthr[pre.ne] = verhulst_thresholds(P.act[P.verhulst_act[0]], Kc[d], nnew[j]);
                    } else if (crn[j] != kNoRun) {
                        vthr[pre.ne] = verhulst_thresholds(BB.runs[crn[j]].act[P.verhulst_act[0]], Kc[d], nnew[j]);
                    }
                }
                if (P.has_move) necm[pre.ne] = cmove[d];
                // tiles begin at the first cell starting at or after t * kTileAgents
                // (rows past the capacity are never written: the step fails with kErrCapacity)
                const uint32_t e = min(pre.n + nnew[j], P.capacity);
                if (pre.n % (uint32_t)kTileAgents == 0u && pre.n <= P.capacity) {
                    new_tile_first[pre.n / kTileAgents] = pre.ne;
                }
                for (uint32_t t = pre.n / kTileAgents + 1u; t * (uint32_t)kTileAgents <= e; t++) {
                    new_tile_first[t] = pre.ne + 1u;
                }
                if (nnew[j] > (uint32_t)kMaxCellBig) set_error(rs, kErrCellTooLarge, (uint32_t)d);
                cmax = max(cmax, nnew[j]);
            }
            pre.n += nnew[j];
            pre.b += bth[j];
            pre.ne += (nnew[j] > 0u) ? 1u : 0u;
        }
    }
    // the next step's form depends on cells above kMaxCellWarp (and kMaxCell)
    cmax = __reduce_max_sync(FULL_MASK, cmax);
    if (lane == 0 && cmax > (uint32_t)kMaxCellWarp) atomicMax(&rs->max_cell, cmax);
}

// ----------------------------------------------------------------- scatter
// The last CTA of a step's scatter commits the step: agent and cell counts,
// next ID, statistics, genome free list, the form of the next step (the big
// form applies it).  Every thread of the CTA calls it; `flag` is a shared word.
template <bool BATCH, bool BIG>
__device__ __forceinline__ void commit_step(const StepConst &P, const BatchBuffers &BB, RunState *__restrict__ rs,
                                            uint32_t *flag) {
    const int tid = threadIdx.x;
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        const uint32_t done = atomicAdd(&rs->scatter_ctas_done, 1u);
        *flag = 0u;
        if (done == gridDim.x - 1) {
            __threadfence();
            rs->scatter_ctas_done = 0u;
            if (atomicAdd(&rs->error, 0u) != 0u) {   // a CTA failed: keep the old table
                rs->dead_count = 0u;
            } else {
                *flag = 1u;
            }
        }
    }
    __syncthreads();
    const uint32_t step = (uint32_t)rs->step;
    if (BATCH && *flag) {
        // per run: next ID after this step's births; the next ring slot starts at zero
        const uint32_t sl = step % kBatchRing, sn = (step + 1u) % kBatchRing;
        for (int r = tid; r < BB.nruns; r += blockDim.x) {
            BB.rnext[r] += (int64_t)BB.rstat[((size_t)r * kBatchRing + sl) * 4 + 1];
            uint4 *z = reinterpret_cast<uint4 *>(BB.rstat + ((size_t)r * kBatchRing + sn) * 4);
            *z = make_uint4(0u, 0u, 0u, 0u);
        }
        __threadfence();
    }
    __syncthreads();
    if (tid == 0 && *flag) {
        rs->stats[step % kStatsRing][0] = rs->new_n_agents;
        unsigned long long *nx = rs->stats[(step + 1u) % kStatsRing];
        nx[0] = 0ull; nx[1] = 0ull; nx[2] = 0ull; nx[3] = 0ull;
        rs->n_agents = rs->new_n_agents;
        rs->n_nonempty = rs->new_n_nonempty;
        rs->form_next = step_form(rs->max_cell, rs->new_n_agents, rs->new_n_nonempty, P.dense_cell);
        if (BIG) rs->form = rs->form_next;
        rs->max_cell = 0u;
        rs->next_id += (int64_t)rs->births;
        rs->birth_log_n += rs->births;
        rs->action_tiles = 0u;
        rs->scatter_tiles = 0u;
        if (P.genome_words > 0) {
            const uint32_t b = rs->births, nf = rs->nfree;
            rs->hwm += (b > nf) ? b - nf : 0u;
            rs->nfree = (nf > b ? nf - b : 0u) + rs->dead_count;
            rs->dead_count = 0u;
            rs->genome_step = (int32_t)step;
        }
        if (!BATCH && P.age_from_birth) rs->age_derived = 1u;
        rs->step = (int32_t)(step + 1u);
        __threadfence();
    }
}

template <int TM, int TT>
struct ScatterSmemT {
    uint32_t sb[kTileCells];       // first row of the cell's stayers in the next table
    uint32_t bb[kTileCells];       // first row of its newborns
    uint32_t bid[kTileCells];      // birth number of its first newborn
    uint32_t ob[kTileCells][6];    // first row of its movers, per neighbour slot
    int64_t bmid[TM];              // the tile's mothers (dense): IDs,
    uint32_t brow[TM];             // ... row | local cell << 16,
    int32_t bfr[TM];               // ... their mates' rows,
    uint16_t brk[TM];              // ... their birth ranks in the cell
    uint32_t crn[kTileCells];      // batches: run of each cell
    float cft[kTileCells];         // batches: time of the cell's run
    uint32_t nb[2];                // mothers of the tile, by parity of the CTA's tile count
    uint32_t last;
};

template <bool BATCH, bool BIG>
__global__ void __launch_bounds__(Tile<BIG>::kThreads, BIG ? 1 : 4)
k_scatter(const StepConst P, const BatchBuffers BB, RunState *__restrict__ rs,
          const uint32_t *__restrict__ nonempty, const uint32_t *__restrict__ ne_start,
          const uint32_t *__restrict__ tile_first,
          const int64_t *__restrict__ id, const float *__restrict__ birth,
          const float *__restrict__ age, const float *__restrict__ lastb,
          const uint32_t *__restrict__ outc, const int32_t *__restrict__ father,
          const uint16_t *__restrict__ brank, const uint8_t *__restrict__ nnbr,
          const uint32_t *__restrict__ sbase, const uint32_t *__restrict__ bbase,
          const uint32_t *__restrict__ bidbase, const uint32_t *__restrict__ obase,
          uint32_t *__restrict__ clsc,
          int64_t *__restrict__ id2, float *__restrict__ birth2, float *__restrict__ age2,
          float *__restrict__ lastb2, uint8_t *__restrict__ meta2,
          int64_t *__restrict__ blog, uint64_t blog_cap,
          const int32_t *__restrict__ gslot, int32_t *__restrict__ gslot2,
          const uint32_t *__restrict__ freelist, uint32_t *__restrict__ freelist2,
          uint32_t *__restrict__ brec) {
    constexpr int TT = Tile<BIG>::kThreads;
    constexpr int TM = Tile<BIG>::kMax;
    extern __shared__ __align__(16) unsigned char qhg_smem[];
    ScatterSmemT<TM, TT> &S = *reinterpret_cast<ScatterSmemT<TM, TT> *>(qhg_smem);
    if (rs->error != 0u) return;   // the state stays as before the step
    // The form of this step is read once per CTA.  The tile and cell forms
    // are launched first; their commit only records the next step's form, and
    // the big form -- launched last -- applies it, from its last CTA, whether
    // it ran the step or not, so that no CTA of any form sees the flag change.
    if (threadIdx.x == 0) S.last = rs->form;
    __syncthreads();
    if (S.last != (BIG ? kFormBig : kFormTile)) {
        if (BIG && threadIdx.x == 0) {
            __threadfence();
            if (atomicAdd(&rs->scatter_ctas_done, 1u) == gridDim.x - 1) {
                rs->scatter_ctas_done = 0u;
                rs->form = rs->form_next;
                __threadfence();
            }
        }
        return;
    }
    __syncthreads();
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int32_t step = rs->step;
    const float fT = (float)step;
    const int64_t next_id = rs->next_id;
    const uint64_t blog_base = rs->birth_log_n;
    const uint32_t N = rs->n_agents;
    const uint32_t cap = P.capacity;
    const uint32_t ntiles = (N + kTileAgents - 1) / kTileAgents;
    constexpr int RA = TM / TT;
    // genome slots (SPopulation::recycleDeadSpaceNew, core/SPopulation.cpp:596-724):
    // newborns take the slots freed by the previous step's deaths, in birth
    // order, then never used slots; this step's deaths free theirs for the
    // next step, so a newborn never overwrites a parent of the same step
    const bool genetics = P.genome_words > 0;
    const uint32_t births = rs->births;
    const uint32_t nfree = rs->nfree;
    const uint32_t hwm = rs->hwm;
    const uint32_t carry = nfree > births ? nfree - births : 0u;
    if (genetics) {
        for (uint32_t q = blockIdx.x * blockDim.x + tid; q < carry; q += gridDim.x * blockDim.x) {
            freelist2[q] = freelist[births + q];
        }
    }
    if (tid == 0) { S.nb[0] = 0u; S.nb[1] = 0u; }
    // the bounds of the CTA's next tile are loaded one tile ahead
    uint32_t nr0 = 0, nr1 = 0, na0 = 0, na1 = 0;
    if (blockIdx.x < ntiles) {
        nr0 = tile_first[blockIdx.x];
        nr1 = tile_first[blockIdx.x + 1];
        na0 = ne_start[nr0];
        na1 = ne_start[nr1];
    }
    uint32_t par = 0u;   // parity of the tiles this CTA has worked on
    for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const uint32_t r0 = nr0;
        const int nc = (int)(nr1 - r0);
        const uint32_t a0 = na0;
        const int na = (int)(na1 - na0);
        const uint32_t tn = t + gridDim.x;
        if (tn < ntiles) {
            nr0 = tile_first[tn];
            nr1 = tile_first[tn + 1];
        }
        if (nc == 0 || na > TM || nc > kTileCells) {   // reported by k_actions
            if (tn < ntiles) {
                na0 = ne_start[nr0];
                na1 = ne_start[nr1];
            }
            continue;
        }
        uint32_t pc[RA];
        int64_t pid[RA];
        float pb[RA], pa[RA], pl[RA];
        int32_t pg[RA];
#pragma unroll
        for (int j = 0; j < RA; j++) {
            const int i = tid + j * TT;
            pc[j] = 0;
            pg[j] = 0;
            if (i < na) {
                if (genetics) pg[j] = gslot[a0 + i];
                pc[j] = outc[a0 + i];
                pid[j] = id[a0 + i];
                pb[j] = birth[a0 + i];
                pa[j] = P.age_from_birth ? 0.0f : age[a0 + i];
                pl[j] = lastb[a0 + i];
            }
        }
        __syncthreads();   // the previous tile is done with the shared arrays
        for (int lc = tid; lc < nc; lc += TT) {
            const uint32_t c = nonempty[r0 + lc];
            S.sb[lc] = sbase[c];
            S.bb[lc] = bbase[c];
            S.bid[lc] = bidbase[c];
            if (BATCH) {
                // birth ranks and IDs count within the run
                const uint32_t r = BB.crun[c];
                const BatchRun &R = BB.runs[r];
                S.crn[lc] = r;
                S.bid[lc] = bidbase[c] - bidbase[R.cell0];
                S.cft[lc] = (float)(step - R.step0);
            }
            // all six slots (unused ones hold stale values that no agent reads),
            // so that the loads do not wait for the neighbour count
#pragma unroll
            for (int k = 0; k < 6; k++) S.ob[lc][k] = obase[(size_t)c * 6 + k];
            // the class counts are consumed: clear them for the next step
            uint4 *z = reinterpret_cast<uint4 *>(clsc + (size_t)c * kCls);
            z[0] = make_uint4(0u, 0u, 0u, 0u);
            z[1] = make_uint4(0u, 0u, 0u, 0u);
        }
        // the tile's mothers to a dense list, with their mates and birth ranks
        // (written by k_actions), read while the cell bases are on their way
        if (tid == 0) S.nb[par ^ 1u] = 0u;   // the counter of the next tile
#pragma unroll
        for (int j = 0; j < RA; j++) {
            const int i = tid + j * TT;
            if (__all_sync(FULL_MASK, i >= na)) break;
            const bool mo = i < na && (pc[j] & kOutBirth);
            const uint32_t mm = __ballot_sync(FULL_MASK, mo);
            if (mm) {
                uint32_t base = 0;
                if (lane == 0) base = atomicAdd(&S.nb[par], (uint32_t)__popc(mm));
                base = __shfl_sync(FULL_MASK, base, 0);
                if (mo) {
                    const uint32_t q = base + __popc(mm & lanemask_lt());
                    const uint32_t row = a0 + (uint32_t)i;
                    S.brow[q] = (uint32_t)i | (((pc[j] >> 8) & 511u) << 16);
                    S.bfr[q] = father[row];
                    S.brk[q] = brank[row];
                    S.bmid[q] = pid[j];
                }
            }
        }
        // the next tile's first row and end, requested while this tile works
        if (tn < ntiles) {
            na0 = ne_start[nr0];
            na1 = ne_start[nr1];
        }
        __syncthreads();
        // every agent to its cell's class base + its rank in the class (from
        // k_actions): survivors and movers into the next table
#pragma unroll
        for (int j = 0; j < RA; j++) {
            const int i = tid + j * TT;
            if (__all_sync(FULL_MASK, i >= na)) break;
            const bool in_tile = i < na;
            const uint32_t code = pc[j];
            const int k = code & 7;
            if (genetics && __any_sync(FULL_MASK, in_tile && k == 0)) {
                // the genome slot of an agent dying this step goes to the next free list
                const uint32_t q = warp_agg_add(in_tile && k == 0, 0u, &rs->dead_count, 1u);
                if (in_tile && k == 0) {
                    if (carry + q < P.genome_capacity) freelist2[carry + q] = (uint32_t)pg[j];
                    else set_error(rs, kErrInternal, 5u);
                }
            }
            if (!in_tile || k == 0) continue;
            const int lc = (int)((code >> 8) & 511u);
            if (lc >= nc) {   // inconsistent outcome word: record, never index past the tile
                set_error(rs, kErrInternal, 7u);
                continue;
            }
            const uint32_t dst = ((k == 1) ? S.sb[lc] : S.ob[lc][k - 2]) + (code >> 17);
            if (dst >= cap) {   // inconsistent bases: record, never write out of range
                set_error(rs, kErrInternal, 3u);
            } else {
                const float fb = pb[j];
                id2[dst] = pid[j];
                birth2[dst] = fb;
                lastb2[dst] = pl[j];
                if (BATCH || !P.age_from_birth) age2[dst] = P.age_from_birth ? __fsub_rn(S.cft[lc], fb) : pa[j];
                meta2[dst] = (uint8_t)(((code & kOutGender) ? kMetaGender : 0) |
                                       ((code & kOutFertile) ? kMetaFertile : 0));
                if (genetics) gslot2[dst] = pg[j];
            }
        }
        __syncthreads();
        // newborns, one thread per mother (SPopulation::createAgentAtIndex,
        // core/SPopulation.cpp:880-900): gender = (uchar)(2 * wrandd()) from the
        // mother's birth stream, females start FERTILE
        const uint32_t nbt = S.nb[par];
        for (uint32_t q = tid; q < nbt; q += TT) {
            const int i = (int)(S.brow[q] & 0xffffu);
            const uint32_t row = a0 + (uint32_t)i;
            const int lc = (int)(S.brow[q] >> 16);
            const uint32_t rk = S.brk[q];
            const int32_t fr = S.bfr[q];
            const uint32_t dst = (lc < nc ? S.bb[lc] : cap) + rk;
            const bool ok = dst < cap && fr >= 0 && (uint32_t)fr < N;
            if (!ok) {
                set_error(rs, kErrInternal, 4u);
                continue;
            }
            const int64_t mid = S.bmid[q];
            uint64_t sd = P.seed;
            int32_t st = step;
            float ft = fT;
            int64_t nid = next_id;
            if (BATCH) {
                const BatchRun &R = BB.runs[S.crn[lc]];
                sd = R.seed;
                st = step - R.step0;
                ft = S.cft[lc];
                nid = BB.rnext[S.crn[lc]];
            }
            const uint32_t u = run_block<BATCH>(P, sd, (uint32_t)st, mid, kStreamBirth).v[0];
            const uint8_t g = (uint8_t)(u >> 31);
            const int64_t baby = nid + (int64_t)(S.bid[lc] + rk);
            id2[dst] = baby;
            birth2[dst] = ft;
            lastb2[dst] = 0.0f;
            if (BATCH || !P.age_from_birth) age2[dst] = 0.0f;
            meta2[dst] = (uint8_t)(g ? kMetaGender : kMetaFertile);
            if (genetics) {
                const uint32_t gr = S.bid[lc] + rk;   // birth rank of the step
                const uint32_t bs = gr < nfree ? freelist[gr] : hwm + (gr - nfree);
                if (bs >= P.genome_capacity) {
                    set_error(rs, kErrCapacity, bs);
                } else {
                    gslot2[dst] = (int32_t)bs;
                    uint32_t *br = brec + (size_t)gr * 5;
                    br[0] = (uint32_t)gslot[row];
                    br[1] = (uint32_t)gslot[fr];
                    br[2] = bs;
                    br[3] = (uint32_t)(uint64_t)mid;
                    br[4] = (uint32_t)((uint64_t)mid >> 32);
                }
            }
            if (P.log_births) {
                const uint64_t li = blog_base + (uint64_t)(S.bid[lc] + rk);
                if (li < blog_cap) {
                    blog[li * 3 + 0] = baby;
                    blog[li * 3 + 1] = mid;
                    blog[li * 3 + 2] = id[fr];
                }
            }
        }
        par ^= 1u;
    }
    commit_step<BATCH, BIG>(P, BB, rs, &S.last);
}

// ------------------------------------------------------ warp-per-cell kernels
// The cell form of a step (non-empty cells of kDenseCell agents or more on
// average, none above kMaxCellWarp): each warp works on its own cells with
// warp-level synchronisation only.  The action kernel takes pairs of
// adjacent cells (2u, 2u + 1) as units, the scatter single cells; the warps
// of the grid take the units in turn (warp g: g, g + G, ...; G the warps of
// the grid).
constexpr int kCellThreads = 256;
constexpr int kCellWarps = kCellThreads / 32;

// per-warp shared memory of k_actions_cell: a group of up to kGroupCells
// adjacent non-empty cells holding up to kMaxCellWarp agents together, rows
// numbered within the group
constexpr int kGroupCells = 2;
struct CellWarpSmem {
    uint32_t fk[kMaxCellWarp];       // FERTILE members: low words of their IDs, in each cell's rows
                                     // (females from the cell's first row up, males from its last row down)
    uint16_t frow[kMaxCellWarp];     // ... their rows
    // the deferred moves' direction draws live from the first pass to the
    // deferred-move pass, the ID-ordered positions and the picks from the ID
    // ranks on: they share their room
    union {
        uint32_t mu2[kMaxCellWarp];  // direction draws of the queued moves (mq)
        struct {
            uint16_t sidx[kMaxCellWarp];  // list positions in ID order, in the same places as the lists
            uint16_t pick[kMaxCellWarp];  // pick values of a cell's smaller side (ID order), from the cell's first row
        } lp;
    };
    int16_t mate[kMaxCellWarp];      // mate's row of each row, -1 none
    uint16_t st[kMaxCellWarp];       // per row: state before the pairing (agent_state), then the outcome byte
    uint32_t odie[kMaxCellWarp / 32];  // OldAgeDeath decided in advance: bit per row, set = dies
    uint16_t oq[kMaxCellWarp];       // rows inside the OldAgeDeath age window, in a dense queue (then mothers)
    uint16_t mq[kMaxCellWarp];       // rows whose move draw passed (deferred moves), in a dense queue (then
                                     // the mothers' list positions)
    uint32_t cnt[kGroupCells][8];    // class counts: [0] stay, [1..6] movers per neighbour slot
    // WeightedMove thresholds of each cell (slots 0-5) as 32-bit values: a
    // threshold of 2^32 (no draw reaches it) is kept as 0xffffffff and its
    // slot marked in wnever (see agent_state)
    __align__(16) uint32_t wt32[kGroupCells][8];
    uint32_t wnever[kGroupCells];
    CellView cv[kGroupCells];        // Verhulst thresholds and move word of each cell
    uint32_t run[kGroupCells];       // batches: run of each cell
};

// four CTAs per SM (64 registers): five fit in shared memory and a
// specialised program fits in 48 registers without spills, but then runs
// 10 % more instructions and measured slower
template <int PROG, bool BATCH>
__global__ void __launch_bounds__(kCellThreads, 4)
k_actions_cell(const StepConst P, const BatchBuffers BB, RunState *__restrict__ rs,
               const uint32_t *__restrict__ nonempty, const uint32_t *__restrict__ ne_start,
               const int64_t *__restrict__ id, const float *__restrict__ birth,
               const float *__restrict__ age, const float *__restrict__ lastb,
               const uint8_t *__restrict__ meta,
               const ulonglong2 *__restrict__ vthr, const uint64_t *__restrict__ wthr,
               const uint32_t *__restrict__ necm,
               uint32_t *__restrict__ outc, int32_t *__restrict__ father, uint32_t *__restrict__ clsc) {
    extern __shared__ __align__(16) unsigned char qhg_smem[];
    __shared__ uint32_t red[kCellWarps];
    CellWarpSmem &W = reinterpret_cast<CellWarpSmem *>(qhg_smem)[threadIdx.x >> 5];
    if (rs->error != 0u) return;   // an earlier kernel failed: keep the state
    if (rs->form != kFormCell) return;   // another form runs this step
    // OldAgeDeath of a specialised program is decided before the other
    // actions, in the same dense draw pass as the pairing picks
    constexpr int kOad = prog_oad_index(PROG);
    constexpr bool kEarlyOad = kOad >= 0;
    // a specialised program reads each agent once: its actions run with the
    // FERTILE lists (keeping both outcomes where the outcome depends on a
    // mate), the outcome is settled after the pairing
    constexpr bool kOnePass = PROG > 0;
    const int lane = threadIdx.x & 31;
    const uint32_t lt = lanemask_lt();
    const int32_t step = rs->step;
    const float fT = (float)step;
    // the table's ages: derived from birth times once a step of a single run has run
    const bool derived = !BATCH && rs->age_derived != 0u;
    const float fTprev = (float)(step - 1);
    const uint32_t nne = rs->n_nonempty;
    uint32_t cnt_births = 0, cnt_deaths = 0, cnt_moves = 0;
    // units of work: pairs of adjacent non-empty cells (2u, 2u + 1), taken by
    // the warps in turn; their bounds are loaded one unit ahead
    const uint32_t units = (nne + 1u) / 2u;
    const uint32_t U = gridDim.x * kCellWarps;
    uint32_t u = blockIdx.x * kCellWarps + (threadIdx.x >> 5);
    uint32_t e0 = 0, e1 = 0, e2 = 0;
    if (u < units) {
        e0 = ne_start[2u * u];
        e1 = ne_start[min(2u * u + 1u, nne)];
        e2 = ne_start[min(2u * u + 2u, nne)];
    }
    for (; u < units; u += U) {
        const uint32_t b0 = e0, b1 = e1, b2 = e2;
        const uint32_t un = u + U;
        if (un < units) {
            e0 = ne_start[2u * un];
            e1 = ne_start[min(2u * un + 1u, nne)];
            e2 = ne_start[min(2u * un + 2u, nne)];
        }
        const int ncu = (2u * u + 1u < nne) ? 2 : 1;   // cells of the unit
        // both cells in one group when their rows fit, else one after the other
        const bool together = ncu == 2 && (b2 - b0) <= (uint32_t)kMaxCellWarp;
        const int ngroups = together ? 1 : ncu;
        for (int gi = 0; gi < ngroups; gi++) {
            const int nc = together ? 2 : 1;                 // cells of the group
            const uint32_t r0 = 2u * u + (uint32_t)gi;       // its first cell's slot in the non-empty list
            const uint32_t s = (gi == 0) ? b0 : b1;          // its first row
            const int n = (int)(((together || ncu == 1 || gi == 1) ? b2 : b1) - s);
            const int cs1 = (nc == 2) ? (int)(b1 - b0) : n;  // first row of the second cell
            if (n > kMaxCellWarp) {   // cannot happen: such steps run a tile form
                if (lane == 0) set_error(rs, kErrCellTooLarge, r0);
                continue;
            }
            // ---- the cells: index, Verhulst thresholds (LinearBirth / LinearDeath
            // ::initialize, actions/LinearBirth.cpp:90-112, actions/LinearDeath.cpp:92-122,
            // computed by the previous step's cell scan), move word, WeightedMove
            // thresholds (lane 8 lc + q holds slot q of cell lc)
            {
                const int lc = lane >> 3, q = lane & 7;
                bool never = false;
                if (lc < nc) {
                    const uint32_t c = nonempty[r0 + (uint32_t)lc];
                    if (P.has_wmove) {
                        const uint64_t w = (q < 6) ? wthr[(size_t)c * 6 + q] : (1ull << 32);
                        never = (w >> 32) != 0ull;
                        W.wt32[lc][q] = never ? 0xffffffffu : (uint32_t)w;
                    }
                    if (q == 6) {
                        ulonglong2 v = make_ulonglong2(0ull, 0ull);
                        uint32_t cm = 0u;
                        if (P.n_verhulst > 0) v = vthr[r0 + (uint32_t)lc];
                        if (P.has_move) cm = necm[r0 + (uint32_t)lc];
                        CellView cv;
                        cv.tk = (uint32_t)(v.x >> 62);
                        cv.tb = v.x & ((1ull << 62) - 1ull);
                        cv.td = v.y;
                        cv.nn = cm & 7u;
                        cv.vm = (cm >> 8) & 63u;
                        cv.wv = (cm >> 24) & 63u;
                        cv.wf = (cm >> 16) & 1u;
                        cv.c = c;
                        W.cv[lc] = cv;
                        if (BATCH) W.run[lc] = BB.crun[c];
                    }
                    if (q == 7) {
                        W.cnt[lc][0] = W.cnt[lc][1] = W.cnt[lc][2] = W.cnt[lc][3] = 0u;
                        W.cnt[lc][4] = W.cnt[lc][5] = W.cnt[lc][6] = W.cnt[lc][7] = 0u;
                    }
                }
                const uint32_t nv = __ballot_sync(FULL_MASK, never && q < 6);
                if (lane < kGroupCells) W.wnever[lane] = (nv >> (8 * lane)) & 63u;
            }
            __syncwarp();
            // a run that leaves the batch drops its agents (they take no part in pairing)
            bool keep0 = true, keep1 = true;
            if (BATCH) {
                keep0 = BB.runs[W.run[0]].active != 0u;
                keep1 = nc == 2 && BB.runs[W.run[nc == 2 ? 1 : 0]].active != 0u;
            }
            // ---- RandomPair::findMates (actions/RandomPair.cpp:146-270): FERTILE
            // lists of each cell, ranked by ID; the members of the smaller side
            // pick, in ID order, each pick drawn from the pairing stream of the
            // picking member.  With an early OldAgeDeath, the agents inside its
            // age window are marked.
            int nF0 = 0, nM0 = 0, nF1 = 0, nM1 = 0, nq = 0, nmv = 0;
            bool wide = false;
            if (kOnePass || P.has_pair || kEarlyOad) {
                for (int b = 0; b < n; b += 32) {
                    uint32_t mu2 = 0u;
                    const int row = b + lane;
                    const bool valid = row < n;
                    const int lc = row >= cs1 ? 1 : 0;
                    const bool kp = valid && (lc ? keep1 : keep0);
                    uint8_t m8 = 0;
                    int64_t xid = 0;
                    float fb = 0.0f, fa = 0.0f, fl = 0.0f;
                    if (kp) {
                        const uint32_t g = s + (uint32_t)row;
                        if (kOnePass || P.has_pair) {
                            m8 = meta[g];
                            xid = id[g];
                        }
                        if (kOnePass || kEarlyOad) fb = birth[g];
                        if (kOnePass) {
                            if (P.reads_age) fa = derived ? __fsub_rn(fTprev, fb) : age[g];
                            fl = lastb[g];
                        }
                    }
                    const bool fert = P.has_pair && (m8 & kMetaFertile) != 0;
                    const bool male = (m8 & kMetaGender) != 0;
                    const int64_t x = fert ? xid : 0;
                    uint32_t stt = 0u;
                    if (kOnePass && kp) {
                        const BatchRun *R = BATCH ? BB.runs + W.run[lc] : nullptr;
                        stt = agent_state<PROG, BATCH, !BATCH>(P, R, step, fT, xid, m8, fb, fa, fl, W.cv[lc],
                                                               W.wt32[lc], W.wnever[lc], &mu2);
                        W.st[row] = (uint16_t)stt;
                    }
                    if (kOnePass && !BATCH) {
                        // deferred moves: queue the rows whose move draw passed
                        const bool mv = (stt & kStMoveDraw) != 0u;
                        const uint32_t mm = __ballot_sync(FULL_MASK, mv);
                        if (mv) {
                            const int qp = nmv + __popc(mm & lt);
                            W.mq[qp] = (uint16_t)row;
                            W.mu2[qp] = mu2;
                        }
                        nmv += __popc(mm);
                    }
                    if (P.has_pair && valid) W.mate[row] = -1;
                    const uint32_t f0 = __ballot_sync(FULL_MASK, fert && !male && lc == 0);
                    const uint32_t f1 = __ballot_sync(FULL_MASK, fert && !male && lc == 1);
                    const uint32_t m0 = __ballot_sync(FULL_MASK, fert && male && lc == 0);
                    const uint32_t m1 = __ballot_sync(FULL_MASK, fert && male && lc == 1);
                    if (fert) {
                        int pos;
                        if (lc == 0) pos = male ? cs1 - 1 - (nM0 + __popc(m0 & lt)) : nF0 + __popc(f0 & lt);
                        else pos = male ? n - 1 - (nM1 + __popc(m1 & lt)) : cs1 + nF1 + __popc(f1 & lt);
                        W.fk[pos] = (uint32_t)(uint64_t)x;
                        W.frow[pos] = (uint16_t)row;
                    }
                    wide |= __any_sync(FULL_MASK, ((uint64_t)x >> 32) != 0ull);
                    nF0 += __popc(f0);
                    nF1 += __popc(f1);
                    nM0 += __popc(m0);
                    nM1 += __popc(m1);
                    if (kEarlyOad) {
                        bool inw = false;
                        if (kp) {
                            if (kOnePass) {
                                // inside the window and alive after Verhulst in some case
                                const bool may_live = !(stt & kStDeadU) || ((stt & kStMateDep) && !(stt & kStDeadM));
                                inw = ((stt >> kStOad) & 3u) == 2u && may_live;
                            } else {
                                const BatchRun *R = BATCH ? BB.runs + W.run[lc] : nullptr;
                                const ActionConst &A = BATCH ? R->act[kOad] : P.act[kOad];
                                const float fTR = BATCH ? (float)(step - R->step0) : fT;
                                const float fa2 = __fsub_rn(fTR, fb);
                                inw = !(fa2 <= A.age_lo) && !(fa2 > A.age_hi);
                            }
                        }
                        const uint32_t qm = __ballot_sync(FULL_MASK, inw);
                        if (inw) W.oq[nq + __popc(qm & lt)] = (uint16_t)row;
                        nq += __popc(qm);
                        if (lane == 0) W.odie[b >> 5] = 0u;
                    }
                }
                __syncwarp();
            }
            // per cell: the list regions, the smaller (picking) side and the larger one
            const bool pairs0 = nF0 > 0 && nM0 > 0, pairs1 = nF1 > 0 && nM1 > 0;
            const bool fs0 = nF0 <= nM0, fs1 = nF1 <= nM1;
            const int m0 = pairs0 ? (fs0 ? nF0 : nM0) : 0, m1 = pairs1 ? (fs1 ? nF1 : nM1) : 0;
            const uint32_t nL0 = (uint32_t)(fs0 ? nM0 : nF0), nL1 = (uint32_t)(fs1 ? nM1 : nF1);
            const int sb0 = fs0 ? 0 : cs1 - nM0, sb1 = fs1 ? cs1 : n - nM1;     // smaller side in sidx
            const int lb0 = fs0 ? cs1 - nM0 : 0, lb1 = fs1 ? n - nM1 : cs1;     // larger side
            // ---- the directions of the deferred moves, one lane per queued row
            if (kOnePass && !BATCH) {
                constexpr int iMv = prog_index(PROG, kRandomMove, kWeightedMove);
                constexpr bool kWeightedMv = PROG > 0 && prog_act(PROG, iMv > 0 ? iMv : 0) == kWeightedMove;
                for (int t = lane; t < nmv; t += 32) {
                    const int row = W.mq[t];
                    const int lc = row >= cs1 ? 1 : 0;
                    W.st[row] = (uint16_t)(W.st[row] | move_direction<kWeightedMv>(W.cv[lc], W.wt32[lc], W.wnever[lc],
                                                                                   W.mu2[t]));
                }
                __syncwarp();
            }
            // ---- ID ranks of every list entry within its own list, one pass over
            // both cells: entry k goes to sidx[region + rank].  IDs are compared by
            // their low words while all high words are zero, else in full.
            const int nr0 = pairs0 ? nF0 + nM0 : 0;
            const int nr = nr0 + (pairs1 ? nF1 + nM1 : 0);
            for (int t0 = 0; t0 < nr; t0 += 32) {
                const int t = t0 + lane;
                if (t < nr) {
                    const int lc = t >= nr0 ? 1 : 0;
                    const int tt = t - (lc ? nr0 : 0);
                    const int nFl = lc ? nF1 : nF0, nMl = lc ? nM1 : nM0;
                    const bool male = tt >= nFl;
                    const int bse = male ? (lc ? n : cs1) - nMl : (lc ? cs1 : 0);
                    const int cnt = male ? nMl : nFl;
                    const int k = bse + (male ? tt - nFl : tt);
                    int r = 0;
                    if (!wide) {
                        const uint32_t x = W.fk[k];
                        int j = 0;
                        for (; j + 4 <= cnt; j += 4) {
                            r += (W.fk[bse + j] < x ? 1 : 0) + (W.fk[bse + j + 1] < x ? 1 : 0) +
                                 (W.fk[bse + j + 2] < x ? 1 : 0) + (W.fk[bse + j + 3] < x ? 1 : 0);
                        }
                        for (; j < cnt; j++) r += (W.fk[bse + j] < x) ? 1 : 0;
                    } else {
                        const int64_t x = id[s + W.frow[k]];
                        for (int j = 0; j < cnt; j++) r += (id[s + W.frow[bse + j]] < x) ? 1 : 0;
                    }
                    W.lp.sidx[bse + r] = (uint16_t)k;
                }
            }
            __syncwarp();
            // ---- one dense pass of draws: pick j of a cell (j < m) takes the
            // pick[j]-th still unpaired member of its larger side, pick[j] =
            // (int)wrandr(0, nL - j); then the OldAgeDeath draws of the agents in
            // its window: age > M + wrandr(1 - U*M, 1 + U*M) (actions/OldAgeDeath.cpp:57-60)
            const int np = m0 + m1;
            for (int t0 = 0; t0 < np + nq; t0 += 32) {
                const int t = t0 + lane;
                if (t < np + nq) {
                    // one Philox block per lane, from the picking member's pairing
                    // stream or the old agent's action stream
                    int64_t x;
                    uint32_t blk, wd = 0u;
                    int row = 0, lc, j = 0;
                    if (t < np) {
                        lc = t >= m0 ? 1 : 0;
                        j = t - (lc ? m0 : 0);
                        const int pos = W.lp.sidx[(lc ? sb1 : sb0) + j];
                        x = wide ? id[s + W.frow[pos]] : (int64_t)W.fk[pos];
                        blk = kStreamPair;
                    } else {
                        // the (t - np)-th marked row
                        row = W.oq[t - np];
                        lc = row >= cs1 ? 1 : 0;
                        x = id[s + row];
                        constexpr uint32_t w = prog_window(PROG, kOad > 0 ? kOad : 0);
                        blk = kStreamActions + (w >> 2);
                        wd = w & 3u;
                    }
                    const BatchRun *R = BATCH ? BB.runs + W.run[lc] : nullptr;
                    const uint64_t sd = BATCH ? R->seed : P.seed;
                    const int32_t stR = BATCH ? step - R->step0 : step;
                    const Draw4 d4 = run_block<BATCH>(P, sd, (uint32_t)stR, x, blk);
                    if (t < np) {
                        W.lp.pick[(lc ? cs1 : 0) + j] =
                            (uint16_t)(((uint64_t)((lc ? nL1 : nL0) - (uint32_t)j) * (uint64_t)d4.v[0]) >> 32);
                    } else if (kEarlyOad) {
                        const ActionConst &A = BATCH ? R->act[kOad > 0 ? kOad : 0] : P.act[kOad > 0 ? kOad : 0];
                        const float fa = __fsub_rn(BATCH ? (float)stR : fT, birth[s + row]);
                        const uint32_t uu = pick4(d4, wd);
                        const double th = __dmul_rn(__dmul_rn(A.oad_w, (double)uu), 2.3283064365386962890625e-10);
                        const double thr = __dadd_rn(A.oad_M, __dadd_rn(A.oad_a, th));
                        if ((double)fa > thr) atomicOr(&W.odie[row >> 5], 1u << (row & 31));
                    }
                }
            }
            __syncwarp();
            // ---- the member taken by pick j, decoded on its own: start from pick[j]
            // and for i = j-1 down to 0 step over the member pick i took when it
            // lies at or below (the lanes of a pass walk i down together)
            for (int t0 = 0; t0 < np; t0 += 32) {
                const int t = t0 + lane;
                const bool act = t < np;
                const int lc = (act && t >= m0) ? 1 : 0;
                const int j = act ? t - (lc ? m0 : 0) : 0;
                const uint16_t *pk = W.lp.pick + (lc ? cs1 : 0);
                uint32_t p = act ? pk[j] : 0u;
                const int top = __reduce_max_sync(FULL_MASK, (uint32_t)j);
                for (int k = top - 1; k >= 0; k--) {
                    if (k < j) p += (p >= pk[k]) ? 1u : 0u;
                }
                if (act) {
                    if (p >= (lc ? nL1 : nL0)) {   // cannot happen: every pick finds a free member
                        set_error(rs, kErrInternal, 1u);
                    } else {
                        const int a = W.frow[W.lp.sidx[(lc ? sb1 : sb0) + j]];
                        const int bb = W.frow[W.lp.sidx[(lc ? lb1 : lb0) + (int)p]];
                        W.mate[a] = (int16_t)bb;
                        W.mate[bb] = (int16_t)a;
                    }
                }
            }
            __syncwarp();
            // ---- every agent's outcome (a specialised program: settled from its
            // state and its mate; otherwise every action in execution order), then
            // the outcome word with the agent's rank in its cell's class
            uint32_t births0 = 0, births1 = 0, dm0 = 0, dm1 = 0;
            for (int b = 0; b < n; b += 32) {
                const int row = b + lane;
                const bool valid = row < n;
                const int lc = row >= cs1 ? 1 : 0;
                uint8_t oc = 0;
                uint32_t mdir = 0u;   // direction of a registered move, kept for the dead
                if (valid) {
                    const uint32_t g = s + (uint32_t)row;
                    if (!(lc ? keep1 : keep0)) {
                        oc = kOutDropped;
                    } else if (kOnePass) {
                        // LinearBirth / LinearDeath with or without a mate, the move
                        // and OldAgeDeath of an agent still alive
                        const uint32_t stt = W.st[row];
                        const int mate = P.has_pair ? W.mate[row] : -1;
                        const bool mated = (stt & kStMateDep) && mate >= 0;
                        const bool bflag = mated && (stt & kStBirthM);
                        bool alive = !(stt & (mated ? kStDeadM : kStDeadU));
                        if (!alive) cnt_deaths++;
                        const uint32_t dir = alive ? (stt & kStDir) : 0u;
                        if (dir) cnt_moves++;
                        mdir = dir;
                        if (kEarlyOad && alive) {
                            const uint32_t o = (stt >> kStOad) & 3u;
                            if (o == 1u || (o == 2u && ((W.odie[b >> 5] >> lane) & 1u))) {
                                alive = false;
                                cnt_deaths++;
                            }
                        }
                        oc = (uint8_t)((alive ? 1u + dir : 0u) | (bflag ? kOutBirth : 0) |
                                       ((stt & kStFert) ? kOutFertile : 0) | ((stt & kStGender) ? kOutGender : 0) |
                                       (dir ? kOutMoved : 0));
                        if (bflag) {
                            father[g] = (int32_t)(s + (uint32_t)mate);
                            cnt_births++;
                        }
                    } else {
                        const BatchRun *R = BATCH ? BB.runs + W.run[lc] : nullptr;
                        const int mate = P.has_pair ? W.mate[row] : -1;
                        const bool odie = kEarlyOad && ((W.odie[b >> 5] >> lane) & 1u);
                        float fa;
                        bool queued = false;
                        oc = agent_outcome<PROG, BATCH, kEarlyOad ? kOadGiven : kOadDraw>(
                            P, R, step, fT, id[g], meta[g], birth[g],
                            P.reads_age ? (derived ? __fsub_rn(fTprev, birth[g]) : age[g]) : 0.0f, lastb[g],
                            mate >= 0, W.cv[lc], wthr, odie, fa, queued, cnt_deaths, cnt_moves, mdir);
                        if (oc & kOutBirth) {
                            father[g] = (int32_t)(s + (uint32_t)mate);
                            cnt_births++;
                        }
                    }
                    W.st[row] = oc;
                }
                const int cls = oc & 7;
                const bool counted = valid && cls > 0;
                const uint32_t slot = counted ? (uint32_t)(cls - 1) : 0u;
                const uint32_t peers = __match_any_sync(FULL_MASK, counted ? ((uint32_t)lc << 3) | slot : 0xffu);
                const uint32_t base = counted ? W.cnt[lc][slot] : 0u;
                __syncwarp();
                if (counted && (peers & lt) == 0u) W.cnt[lc][slot] = base + (uint32_t)__popc(peers);
                // outcome byte | rank in the cell's class << 17 (for the dead, the
                // direction of a move they registered)
                if (valid)
                    outc[s + (uint32_t)row] =
                        (uint32_t)oc | ((counted ? base + (uint32_t)__popc(peers & lt) : mdir) << 17);
                const bool bo = valid && (oc & kOutBirth);
                births0 += __popc(__ballot_sync(FULL_MASK, bo && lc == 0));
                births1 += __popc(__ballot_sync(FULL_MASK, bo && lc == 1));
                if (BATCH) {
                    const bool dd = valid && cls == 0 && !(oc & kOutDropped);
                    const bool mv = valid && (oc & kOutMoved);
                    dm0 += __popc(__ballot_sync(FULL_MASK, dd && lc == 0)) +
                           ((uint32_t)__popc(__ballot_sync(FULL_MASK, mv && lc == 0)) << 16);
                    dm1 += __popc(__ballot_sync(FULL_MASK, dd && lc == 1)) +
                           ((uint32_t)__popc(__ballot_sync(FULL_MASK, mv && lc == 1)) << 16);
                }
                __syncwarp();
            }
            // ---- mothers' birth ranks: births are numbered in (cell, mother ID)
            // order; mothers are FERTILE females, walked in ID order and queued
            // in birth order (rows and list positions; the OldAgeDeath and move
            // queues are free by now)
            uint32_t nmo = 0;
#pragma unroll
            for (int lc = 0; lc < 2; lc++) {
                if ((lc ? births1 : births0) == 0u) continue;
                const int nFl = lc ? nF1 : nF0, cs = lc ? cs1 : 0;
                for (int q0 = 0; q0 < nFl; q0 += 32) {
                    const int q = q0 + lane;
                    bool mo = false;
                    int row = 0, pos = 0;
                    if (q < nFl) {
                        pos = W.lp.sidx[cs + q];
                        row = W.frow[pos];
                        mo = (W.st[row] & kOutBirth) != 0;
                    }
                    const uint32_t mb = __ballot_sync(FULL_MASK, mo);
                    if (mo) {
                        const uint32_t k = nmo + (uint32_t)__popc(mb & lt);
                        W.oq[k] = (uint16_t)row;
                        W.mq[k] = (uint16_t)pos;
                    }
                    nmo += (uint32_t)__popc(mb);
                }
            }
            __syncwarp();
            // ---- the newborns: one lane per mother, in a dense pass.  Gender =
            // (uchar)(2 * wrandd()) from the mother's birth stream
            // (SPopulation::createAgentAtIndex, core/SPopulation.cpp:880-900),
            // the birth rank in the cell (< 128: a cell of the warp-per-cell form
            // holds at most 256 agents) and the gender join the mother's outcome
            // word (bits 8-15 and 16), which the cell scatter reads
            for (int t = lane; t < (int)nmo; t += 32) {
                const int row = W.oq[t];
                const int lc = row >= cs1 ? 1 : 0;
                const uint32_t rk = (uint32_t)t - (lc ? births0 : 0u);
                const int64_t x = wide ? id[s + (uint32_t)row] : (int64_t)W.fk[W.mq[t]];
                const BatchRun *R = BATCH ? BB.runs + W.run[lc] : nullptr;
                const uint32_t u = run_block<BATCH>(P, BATCH ? R->seed : P.seed,
                                                    (uint32_t)(BATCH ? step - R->step0 : step), x, kStreamBirth)
                                       .v[0];
                atomicOr(&outc[s + (uint32_t)row], (rk << 8) | ((u >> 31) << 16));
            }
            // class counts of each cell: stay, movers per neighbour slot, births
            {
                const int lc = lane >> 3, q = lane & 7;
                if (lc < nc) {
                    const uint32_t c = W.cv[lc].c;
                    clsc[(size_t)c * kCls + q] = (q < 7) ? W.cnt[lc][q] : (lc ? births1 : births0);
                    if (BATCH && q == 0) BB.cstat[c] = lc ? dm1 : dm0;   // deaths | registered moves << 16
                }
            }
            __syncwarp();
        }
    }
    // statistics of the step (batches: per run, by the cell scan)
    if (BATCH) return;
    const uint32_t tb_ = block_sum(cnt_births, red);
    const uint32_t td_ = block_sum(cnt_deaths, red);
    const uint32_t tm_ = block_sum(cnt_moves, red);
    if (threadIdx.x == 0 && (tb_ | td_ | tm_)) {
        unsigned long long *st = rs->stats[(uint32_t)step % kStatsRing];
        atomicAdd(&st[1], (unsigned long long)tb_);
        atomicAdd(&st[2], (unsigned long long)td_);
        atomicAdd(&st[3], (unsigned long long)tm_);
    }
}

// ---- rows staged in shared memory by bulk copies (cp.async.bulk with
// completion counted on an mbarrier): a warp copies the rows of its next
// piece of work while it writes out the current one
constexpr int kStageRows = 128;   // rows of one staged piece (a cell, or a part of a larger one)
constexpr uint32_t kStageSpinLimit = 1u << 24;   // polls of a staging wait (with the time limit kWaitLimitNs)

// bytes of one staged column of kStageRows rows of `elem` bytes: room for the
// 16-byte units around an unaligned row range
__host__ __device__ constexpr uint32_t stage_col_bytes(uint32_t elem) { return (uint32_t)kStageRows * elem + 32u; }
// one staging buffer of the scatter: outcome words, IDs, birth times, last
// births, ages (when the table's ages are not derived from birth times),
// genome slots and mates' rows (genetics)
__host__ __device__ inline uint32_t scatter_stage_bytes(bool age_col, bool gslot_col) {
    return stage_col_bytes(4) + stage_col_bytes(8) + 2u * stage_col_bytes(4) + (age_col ? stage_col_bytes(4) : 0u) +
           (gslot_col ? 2u * stage_col_bytes(4) : 0u);
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// one test of the phase, the thread suspended in hardware for up to about
// kStageSuspendNs while the phase is incomplete
constexpr uint32_t kStageSuspendNs = 20000u;
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "r"(kStageSuspendNs)
        : "memory");
    return ok != 0u;
}

// waits for the phase `parity` of an mbarrier to complete; false when the
// wait ran out of polls or time
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
    uint32_t spins = 0;
    const uint64_t t0 = globaltimer_ns();
    while (!mbar_try_wait(bar, parity)) {
        if (++spins > kStageSpinLimit || globaltimer_ns() - t0 > kWaitLimitNs) return false;
    }
    return true;
}

// bulk copy of `bytes` (a multiple of 16) from global to shared memory, both
// 16-byte aligned, counted on `bar`
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// the 16-byte units holding rows [a, a + n) of a column of `elem`-byte
// values: start offset (bytes) and size; the rows begin `head` bytes in
__device__ __forceinline__ void stage_range(uint32_t a, uint32_t n, uint32_t elem, size_t &off, uint32_t &bytes,
                                            uint32_t &head) {
    const size_t lo = (size_t)a * elem, hi = (size_t)(a + n) * elem;
    off = lo & ~(size_t)15;
    bytes = (uint32_t)(((hi + 15) & ~(size_t)15) - off);
    head = (uint32_t)(lo - off);
}

template <bool BATCH>
__global__ void __launch_bounds__(kCellThreads, 4)
k_scatter_cell(const StepConst P, const BatchBuffers BB, RunState *__restrict__ rs,
               const uint32_t *__restrict__ nonempty, const uint32_t *__restrict__ ne_start,
               const int64_t *__restrict__ id, const float *__restrict__ birth,
               const float *__restrict__ age, const float *__restrict__ lastb,
               const uint32_t *__restrict__ outc, const int32_t *__restrict__ father,
               const uint32_t *__restrict__ sbase, const uint32_t *__restrict__ bbase,
               const uint32_t *__restrict__ bidbase, const uint32_t *__restrict__ obase,
               uint32_t *__restrict__ clsc,
               int64_t *__restrict__ id2, float *__restrict__ birth2, float *__restrict__ age2,
               float *__restrict__ lastb2, uint8_t *__restrict__ meta2,
               int64_t *__restrict__ blog, uint64_t blog_cap,
               const int32_t *__restrict__ gslot, int32_t *__restrict__ gslot2,
               const uint32_t *__restrict__ freelist, uint32_t *__restrict__ freelist2,
               uint32_t *__restrict__ brec) {
    extern __shared__ __align__(16) unsigned char qhg_smem[];
    __shared__ uint32_t s_flag;
    __shared__ __align__(8) uint64_t s_bar[kCellWarps][2];
    if (rs->error != 0u) return;   // the state stays as before the step
    // the form of the step is read once per CTA (the big form, launched
    // last, applies the next step's form)
    if (threadIdx.x == 0) s_flag = rs->form;
    __syncthreads();
    if (s_flag != kFormCell) return;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int32_t step = rs->step;
    const float fT = (float)step;
    const int64_t next_id = rs->next_id;
    const uint64_t blog_base = rs->birth_log_n;
    const uint32_t N = rs->n_agents;
    const uint32_t nne = rs->n_nonempty;
    const uint32_t cap = P.capacity;
    const uint32_t G = gridDim.x * kCellWarps;
    // genome slots (SPopulation::recycleDeadSpaceNew, core/SPopulation.cpp:596-724):
    // newborns take the slots freed by the previous step's deaths, in birth
    // order, then never used slots; this step's deaths free theirs for the
    // next step, so a newborn never overwrites a parent of the same step
    const bool genetics = P.genome_words > 0;
    const bool age_col = !P.age_from_birth;
    const uint32_t births = rs->births;
    const uint32_t nfree = rs->nfree;
    const uint32_t hwm = rs->hwm;
    const uint32_t carry = nfree > births ? nfree - births : 0u;
    if (genetics) {
        for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < carry; q += gridDim.x * blockDim.x) {
            freelist2[q] = freelist[births + q];
        }
    }
    // the warp's two staging buffers and their mbarriers
    const uint32_t sbytes = scatter_stage_bytes(age_col, genetics);
    unsigned char *stage0 = qhg_smem + (size_t)warp * 2u * sbytes;
    uint64_t *bar = s_bar[warp];
    if (lane == 0) {
        mbar_init(&bar[0], 1u);
        mbar_init(&bar[1], 1u);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    uint32_t parity = 0u;     // bit b: phase parity of buffer b's next completion
    uint32_t inflight = 0u;   // bit b: copies into buffer b not yet waited for (lane 0's view)

    // copies rows [g, g + cnt) of the staged columns into buffer b (lane 0)
    auto issue = [&](int b, uint32_t g, uint32_t cnt) {
        if (lane != 0) return;
        // earlier reads of the buffer by the warp are ordered before the copy
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        inflight |= 1u << b;
        unsigned char *buf = stage0 + (size_t)b * sbytes;
        size_t off[6];
        uint32_t by[6], hd[6], total = 0u;
        stage_range(g, cnt, 4, off[0], by[0], hd[0]);
        stage_range(g, cnt, 8, off[1], by[1], hd[1]);
        stage_range(g, cnt, 4, off[2], by[2], hd[2]);
        stage_range(g, cnt, 4, off[3], by[3], hd[3]);
        stage_range(g, cnt, 4, off[4], by[4], hd[4]);
        stage_range(g, cnt, 4, off[5], by[5], hd[5]);
        total = by[0] + by[1] + by[2] + by[3] + (age_col ? by[4] : 0u) + (genetics ? 2u * by[5] : 0u);
        mbar_arrive_expect_tx(&bar[b], total);
        unsigned char *d = buf;
        bulk_g2s(d, reinterpret_cast<const unsigned char *>(outc) + off[0], by[0], &bar[b]);
        d += stage_col_bytes(4);
        bulk_g2s(d, reinterpret_cast<const unsigned char *>(id) + off[1], by[1], &bar[b]);
        d += stage_col_bytes(8);
        bulk_g2s(d, reinterpret_cast<const unsigned char *>(birth) + off[2], by[2], &bar[b]);
        d += stage_col_bytes(4);
        bulk_g2s(d, reinterpret_cast<const unsigned char *>(lastb) + off[3], by[3], &bar[b]);
        d += stage_col_bytes(4);
        if (age_col) {
            bulk_g2s(d, reinterpret_cast<const unsigned char *>(age) + off[4], by[4], &bar[b]);
            d += stage_col_bytes(4);
        }
        if (genetics) {
            bulk_g2s(d, reinterpret_cast<const unsigned char *>(gslot) + off[5], by[5], &bar[b]);
            d += stage_col_bytes(4);
            bulk_g2s(d, reinterpret_cast<const unsigned char *>(father) + off[5], by[5], &bar[b]);
        }
    };

    // pieces of work: the warp's cells in turn (cells r, r + G, ...), each in
    // parts of at most kStageRows rows.  The piece being written (cur) and the
    // one being copied (nxt).  Every cell-level load is issued one piece before
    // its use: when cur is its cell's last piece, the next cell's bases and
    // the index and bounds of the cell after it are loaded while cur's rows
    // are written.
    uint32_t r = blockIdx.x * kCellWarps + (uint32_t)warp;
    uint32_t cs = 0, cn = 0;           // cur: cell start row and rows
    int coff = 0;                      // cur: first row of the piece within the cell
    uint32_t ns_ = 0, nn_ = 0;         // bounds of the cell r + G
    uint32_t nc_ = 0;                  // index of the cell r + G
    // cell data of cur's cell
    uint32_t c = 0, sb = 0, bb = 0, bid = 0, ob = 0;
    if (r < nne) {
        cs = ne_start[r];
        cn = ne_start[r + 1] - cs;
        c = nonempty[r];
        if (r + G < nne) {
            ns_ = ne_start[r + G];
            nn_ = ne_start[r + G + 1] - ns_;
            nc_ = nonempty[r + G];
        }
        issue(0, cs, min(cn, (uint32_t)kStageRows));
        sb = sbase[c];
        bb = bbase[c];
        bid = bidbase[c];
        ob = (lane < 6) ? obase[(size_t)c * 6 + lane] : 0u;
    }
    int buf = 0;
    bool failed = false;
    // the next cell's bases, and the index and bounds of the cell after it
    uint32_t nsb = 0, nbb = 0, nbid = 0, nob = 0;
    uint32_t nns = 0, nnn = 0, nnc = 0;
    float ft = fT;
    int64_t nid = next_id;
    while (r < nne) {
        // the next piece: the rest of this cell, or the next cell's first part
        uint32_t xr = r;
        int xoff = coff + kStageRows;
        uint32_t xs = cs, xn = cn;
        if ((uint32_t)xoff >= cn) {
            xr = r + G;
            xoff = 0;
            xs = ns_;
            xn = nn_;
        }
        if (xr < nne) {
            issue(buf ^ 1, xs + (uint32_t)xoff, min(xn - (uint32_t)xoff, (uint32_t)kStageRows));
            if (xr != r) {
                // the next cell's bases in the next table: stayers, newborns
                // (and their birth numbers), movers per neighbour slot (lane
                // k holds slot k); the cell after it
                nsb = sbase[nc_];
                nbb = bbase[nc_];
                nbid = bidbase[nc_];
                nob = (lane < 6) ? obase[(size_t)nc_ * 6 + lane] : 0u;
                if (xr + G < nne) {
                    nns = ne_start[xr + G];
                    nnn = ne_start[xr + G + 1];
                    nnc = nonempty[xr + G];
                }
            }
        }
        if (coff == 0) {
            if (BATCH) {
                // birth ranks and IDs count within the run
                const uint32_t rr = BB.crun[c];
                const BatchRun &R = BB.runs[rr];
                bid -= bidbase[R.cell0];
                ft = (float)(step - R.step0);
                nid = BB.rnext[rr];
            }
            // the class counts are consumed: clear them for the next step
            if (lane < 2) reinterpret_cast<uint4 *>(clsc + (size_t)c * kCls)[lane] = make_uint4(0u, 0u, 0u, 0u);
        }
        // the rows of the piece, staged
        if (!mbar_wait_bounded(&bar[buf], (parity >> buf) & 1u)) {
            if (lane == 0) set_error(rs, kErrTimeout, 0x5ca7u);
            failed = true;
            break;
        }
        parity ^= 1u << buf;
        inflight &= ~(1u << buf);
        const unsigned char *sp = stage0 + (size_t)buf * sbytes;
        const uint32_t g0 = cs + (uint32_t)coff;
        const int pn = min((int)cn - coff, kStageRows);
        const uint32_t h4 = (g0 & 3u) * 4u, h8 = (g0 & 1u) * 8u;   // heads of 4- and 8-byte columns
        const uint32_t *s_outc = reinterpret_cast<const uint32_t *>(sp + h4);
        const int64_t *s_id = reinterpret_cast<const int64_t *>(sp + stage_col_bytes(4) + h8);
        const float *s_birth = reinterpret_cast<const float *>(sp + stage_col_bytes(4) + stage_col_bytes(8) + h4);
        const float *s_lastb =
            reinterpret_cast<const float *>(sp + 2u * stage_col_bytes(4) + stage_col_bytes(8) + h4);
        const float *s_age = reinterpret_cast<const float *>(sp + 3u * stage_col_bytes(4) + stage_col_bytes(8) + h4);
        const int32_t *s_gslot = reinterpret_cast<const int32_t *>(
            sp + (3u + (age_col ? 1u : 0u)) * stage_col_bytes(4) + stage_col_bytes(8) + h4);
        const int32_t *s_father = s_gslot + stage_col_bytes(4) / 4u;
        for (int b = 0; b < pn; b += 32) {
            const int i = b + lane;
            const bool valid = i < pn;
            const uint32_t g = g0 + (uint32_t)i;
            uint32_t code = 0u;
            int64_t x = 0;
            float fb = 0.0f, fa = 0.0f, fl = 0.0f;
            int32_t gs = 0;
            if (valid) {
                code = s_outc[i];
                x = s_id[i];
                fb = s_birth[i];
                if (age_col) fa = s_age[i];
                fl = s_lastb[i];
                if (genetics) gs = s_gslot[i];
            }
            const int k = code & 7;
            const uint32_t obk = __shfl_sync(FULL_MASK, ob, k >= 2 ? k - 2 : 0);
            if (genetics && __any_sync(FULL_MASK, valid && k == 0)) {
                // the genome slot of an agent dying this step goes to the next free list
                const uint32_t q = warp_agg_add(valid && k == 0, 0u, &rs->dead_count, 1u);
                if (valid && k == 0) {
                    if (carry + q < P.genome_capacity) freelist2[carry + q] = (uint32_t)gs;
                    else set_error(rs, kErrInternal, 5u);
                }
            }
            // every survivor to its cell's class base + its rank in the class
            if (valid && k > 0) {
                const uint32_t dst = ((k == 1) ? sb : obk) + (code >> 17);
                if (dst >= cap) {   // inconsistent bases: record, never write out of range
                    set_error(rs, kErrInternal, 3u);
                } else {
                    id2[dst] = x;
                    birth2[dst] = fb;
                    lastb2[dst] = fl;
                    if (BATCH || !P.age_from_birth) age2[dst] = P.age_from_birth ? __fsub_rn(ft, fb) : fa;
                    meta2[dst] = (uint8_t)(((code & kOutGender) ? kMetaGender : 0) |
                                           ((code & kOutFertile) ? kMetaFertile : 0));
                    if (genetics) gslot2[dst] = gs;
                }
            }
            // newborns (SPopulation::createAgentAtIndex, core/SPopulation.cpp:880-900):
            // gender = (uchar)(2 * wrandd()) from the mother's birth stream,
            // females start FERTILE
            if (valid && (code & kOutBirth)) {
                // birth rank and gender from the mother's outcome word; her
                // mate's row only where his genome slot or ID is needed
                const uint32_t rk = (code >> 8) & 255u;
                const int32_t fr = genetics ? s_father[i] : (P.log_births ? father[g] : 0);
                const uint32_t dst = bb + rk;
                if (dst >= cap || fr < 0 || (uint32_t)fr >= N) {
                    set_error(rs, kErrInternal, 4u);
                } else {
                    const int64_t baby = nid + (int64_t)(bid + rk);
                    id2[dst] = baby;
                    birth2[dst] = ft;
                    lastb2[dst] = 0.0f;
                    if (BATCH || !P.age_from_birth) age2[dst] = 0.0f;
                    meta2[dst] = (uint8_t)(((code >> 16) & 1u) ? kMetaGender : kMetaFertile);
                    if (genetics) {
                        const uint32_t gr = bid + rk;   // birth rank of the step
                        const uint32_t bs = gr < nfree ? freelist[gr] : hwm + (gr - nfree);
                        if (bs >= P.genome_capacity) {
                            set_error(rs, kErrCapacity, bs);
                        } else {
                            gslot2[dst] = (int32_t)bs;
                            uint32_t *br = brec + (size_t)gr * 5;
                            // the mate lies in the same cell: in this piece
                            // unless the cell spans several
                            const int fi = fr - (int)g0;
                            br[0] = (uint32_t)gs;
                            br[1] = (uint32_t)((fi >= 0 && fi < pn) ? s_gslot[fi] : gslot[fr]);
                            br[2] = bs;
                            br[3] = (uint32_t)(uint64_t)x;
                            br[4] = (uint32_t)((uint64_t)x >> 32);
                        }
                    }
                    if (P.log_births) {
                        const uint64_t li = blog_base + (uint64_t)(bid + rk);
                        if (li < blog_cap) {
                            blog[li * 3 + 0] = baby;
                            blog[li * 3 + 1] = x;
                            blog[li * 3 + 2] = id[fr];
                        }
                    }
                }
            }
        }
        __syncwarp();   // the buffer is read out before it is copied into again
        // advance: the next piece becomes the current one
        if (xr != r) {
            cs = ns_;
            cn = nn_;
            c = nc_;
            sb = nsb;
            bb = nbb;
            bid = nbid;
            ob = nob;
            ns_ = nns;
            nn_ = nnn - nns;
            nc_ = nnc;
        }
        r = xr;
        coff = xoff;
        buf ^= 1;
    }
    if (failed) {
        // copies still in flight land before the kernel ends (waits bounded again)
        const uint32_t fl = __shfl_sync(FULL_MASK, inflight, 0);
        for (int b = 0; b < 2; b++) {
            if ((fl >> b) & 1u) mbar_wait_bounded(&bar[b], (parity >> b) & 1u);
        }
    }
    commit_step<BATCH, false>(P, BB, rs, &s_flag);
}

// ------------------------------------------------------------- occupancy
// OccTracker::updateCounts / OccHistory::addEntry (core/OccTracker.cpp,
// core/OccHistory.cpp) for one population: a cell's occupation is recorded
// when it first holds an agent (a cell emptied later keeps its entry, as
// OccHistory ignores masks of zero).  Run after a step's commit on the table
// it made (and after an upload on the uploaded one): every non-empty cell
// without an entry gets the step of that table.
__global__ void __launch_bounds__(256)
k_occupancy(const RunState *__restrict__ rs, const uint32_t *__restrict__ nonempty, int32_t *__restrict__ occ,
            const BatchRun *__restrict__ runs, const uint32_t *__restrict__ crun) {
    if (rs->error != 0u) return;   // the step failed: its table was not committed
    const uint32_t n = rs->n_nonempty;
    const int32_t st = rs->step;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const uint32_t c = nonempty[r];
        if (occ[c] < 0) {
            // a batch's cells record the step of their run (0: the table its
            // agents were admitted into)
            occ[c] = runs != nullptr ? st - runs[crun[c]].step0 : st;
        }
    }
}

// --------------------------------------------------------------- MoveStats
// MoveStats::finalize (actions/MoveStats.cpp:183-256) as one thread runs it,
// with the moves in agent-ID order: a move from cell f to cell t offers t the
// values hops[f] + 1 and dist[f] + the f-t distance, taken from the state
// before the step.  MIN keeps per cell the smallest hops and distance and the
// time of the first arrival; FIRST the values of the first arrival (the
// lowest mover ID of the first step that reaches the cell); LAST those of the
// latest arrival (the highest mover ID of the last step with arrivals).
// Every registered move counts, also that of an agent a later action of the
// step killed (its direction is kept in its outcome word).
constexpr int kMsFirst = 0, kMsMin = 1, kMsLast = 2;
constexpr unsigned long long kMsNoDist = 0x7ff0000000000000ull;   // +inf

// the destination slot of a registered move in an outcome word, -1 none
__device__ __forceinline__ int ms_move_slot(uint32_t code) {
    const int cls = (int)(code & 7u);
    if (cls >= 2) return cls - 2;
    if (cls == 0 && (code & kOutMoved)) return (int)((code >> 17) & 7u) - 1;
    return -1;
}

// pass 0: MIN reduces the candidates, FIRST/LAST elect the mover per
// destination; pass 1 (FIRST/LAST): the elected movers write their values.
// One warp per non-empty cell of the step's table; runs after the actions.
template <int MODE, int PASS>
__global__ void __launch_bounds__(256)
k_ms_pick(const RunState *__restrict__ rs, const uint32_t *__restrict__ nonempty,
          const uint32_t *__restrict__ ne_start, const int64_t *__restrict__ id, const uint32_t *__restrict__ outc,
          const int32_t *__restrict__ nbr, const double *__restrict__ D, const int32_t *__restrict__ hops,
          const double *__restrict__ dist, int32_t *__restrict__ chops, unsigned long long *__restrict__ cdist,
          unsigned long long *__restrict__ ckey) {
    if (rs->error != 0u) return;
    const uint32_t n = rs->n_nonempty;
    const int lane = threadIdx.x & 31;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < n; w += warps) {
        const uint32_t f = nonempty[w];
        const uint32_t r0 = ne_start[w], r1 = ne_start[w + 1];
        for (uint32_t r = r0 + (uint32_t)lane; r < r1; r += 32) {
            const int k = ms_move_slot(outc[r]);
            if (k < 0) continue;
            const int32_t t = nbr[(size_t)f * 6 + (size_t)k];
            if (t < 0) continue;
            if (MODE == kMsMin || PASS == 1) {
                const int32_t h = hops[f] + 1;
                const double d = __dadd_rn(dist[f], D[(size_t)f * 6 + (size_t)k]);
                const unsigned long long db = (unsigned long long)__double_as_longlong(d);
                if (MODE == kMsMin) {
                    atomicMin(&chops[t], h);
                    atomicMin(&cdist[t], db);
                } else {
                    const unsigned long long key = (unsigned long long)id[r] + (MODE == kMsLast ? 1ull : 0ull);
                    if (ckey[t] == key) {
                        chops[t] = h;
                        cdist[t] = db;
                    }
                }
            } else if (MODE == kMsFirst) {
                atomicMin(&ckey[t], (unsigned long long)id[r]);
            } else {
                atomicMax(&ckey[t], (unsigned long long)id[r] + 1ull);
            }
        }
    }
}

// After the commit: the candidates into the state, then cleared.  A failed
// step leaves both untouched (its retry offers the same candidates).
template <int MODE>
__global__ void __launch_bounds__(256)
k_ms_merge(const RunState *__restrict__ rs, int C, int32_t *__restrict__ hops, double *__restrict__ dist,
           double *__restrict__ time, int32_t *__restrict__ chops, unsigned long long *__restrict__ cdist,
           unsigned long long *__restrict__ ckey, const BatchRun *__restrict__ runs,
           const uint32_t *__restrict__ crun) {
    if (rs->error != 0u) return;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < C; c += gridDim.x * blockDim.x) {
        const int32_t ch = chops[c];
        if (ch == INT_MAX) continue;
        const uint32_t rr = runs != nullptr ? crun[c] : 0u;
        if (rr == kNoRun) continue;   // a batch cell of no run (never offered a move)
        // the step that made the moves (a batch's cell: in its run's steps)
        const double t = (double)(float)(rs->step - 1 - (runs != nullptr ? runs[rr].step0 : 0));
        const double cd = __longlong_as_double((long long)cdist[c]);
        const int32_t h = hops[c];
        if (MODE == kMsLast || h < 0) {
            hops[c] = ch;
            dist[c] = cd;
            time[c] = t;
        } else if (MODE == kMsMin) {
            if (ch < h) hops[c] = ch;
            if (cd < dist[c]) dist[c] = cd;
        }
        chops[c] = INT_MAX;
        cdist[c] = kMsNoDist;
        ckey[c] = MODE == kMsFirst ? ~0ull : 0ull;
    }
}

// MoveStats state of the cells [c0, c1) before any move: no arrival (-1),
// no candidates, distances zero (k_ms_origins then marks the cells where the
// population starts: hops, distance and time 0, as the reset of a run alone
// leaves its occupied cells)
__global__ void __launch_bounds__(256)
k_ms_fill(uint32_t c0, uint32_t c1, int mode, int32_t *__restrict__ hops, double *__restrict__ dist, double *__restrict__ time,
          int32_t *__restrict__ chops, unsigned long long *__restrict__ cdist, unsigned long long *__restrict__ ckey,
          double *__restrict__ D) {
    for (uint32_t c = c0 + blockIdx.x * blockDim.x + threadIdx.x; c < c1; c += gridDim.x * blockDim.x) {
        hops[c] = -1;
        dist[c] = -1.0;
        time[c] = -1.0;
        chops[c] = INT_MAX;
        cdist[c] = kMsNoDist;
        ckey[c] = mode == kMsFirst ? ~0ull : 0ull;
        for (int k = 0; k < 6; k++) D[(size_t)c * 6 + k] = 0.0;
    }
}

__global__ void __launch_bounds__(256)
k_ms_origins(uint32_t c0, uint32_t c1, const uint32_t *__restrict__ origin, uint32_t norigin,
             int32_t *__restrict__ hops, double *__restrict__ dist, double *__restrict__ time) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < norigin; i += gridDim.x * blockDim.x) {
        const uint32_t c = c0 + origin[i];
        if (c < c1) {
            hops[c] = 0;
            dist[c] = 0.0;
            time[c] = 0.0;
        }
    }
}

// ----------------------------------------------------------------- genomes
// Poisson(1) inverse-CDF thresholds floor(P(K <= k) * 2^32), k = 0..15, exact
__constant__ uint32_t kPoisson1Cdf32[16] = {
    1580030168u, 3160060337u, 3950075421u, 4213413783u, 4279248373u,
    4292415291u, 4294609777u, 4294923276u, 4294962463u, 4294966817u,
    4294967252u, 4294967292u, 4294967295u, 4294967295u, 4294967295u,
    4294967295u};

__device__ __forceinline__ int poisson1(uint32_t u) {
    int k = 0;
    while (k < 16 && u >= kPoisson1Cdf32[k]) k++;
    return k;
}

// BitGeneUtils::makeMultiMask (genes/BitGeneUtils.cpp:90-109) for the
// breaks of one 64-bit block, fed one at a time in draw order.  The
// reference emits the mask's 64 bits from the top, starting with
// 1 - (breaks % 2), and flips the emitted value when the bit index reaches
// 64 - break, taking the breaks from the last one backwards; a break whose
// flip position lies at or before the previous flip (breaks given out of
// ascending order) is never reached, and neither is any break after it.  So
// the flips that happen are those of the longest run at the end of the draw
// order whose values strictly increase (a break at 0 never flips), each
// toggling the low `break` bits: `mask` is the XOR of those toggles, reset
// whenever a break does not exceed the one before it.
struct BlockMask {
    uint64_t mask = 0ull;
    int last = -1;
    int nb = 0;
    __device__ __forceinline__ void add(uint32_t br) {
        const uint64_t m = (1ull << br) - 1ull;   // br in 0..63
        mask = ((int)br > last) ? (mask ^ m) : m;
        last = (int)br;
        nb++;
    }
    // the mask makeMultiMask returns (all ones without breaks)
    __device__ __forceinline__ uint64_t value() const { return ((nb & 1) ? 0ull : ~0ull) ^ mask; }
};

// draw k (the same for every lane) of the newborn's birth stream, lane L
// holding block L
__device__ __forceinline__ uint32_t birth_draw(const Draw4 &d, int k) {
    const int q = k & 3;
    const uint32_t mine = q == 0 ? d.v[0] : (q == 1 ? d.v[1] : (q == 2 ? d.v[2] : d.v[3]));
    return __shfl_sync(FULL_MASK, mine, k >> 2);
}

// Genetics::makeOffspring (actions/Genetics.cpp:285-337), one warp per
// newborn.  Birth stream of the mother: draw 0 gender (k_scatter), 1 and 2
// the strands taken from mother and father, then (Poisson mode) the two
// crossover counts, the mother's and the father's breakpoints, the mutation
// count and the mutation positions.  Lane L builds blocks L and L + 32 of
// both strands of the newborn: strand 0 is strand i1 of the mother crossed
// over at her breaks (BitGeneUtils::crossOver, genes/BitGeneUtils.cpp:116-188:
// before a block, the parity of the breaks in earlier blocks picks the
// strand, inside it the makeMultiMask mask mixes the two), strand 1 the same
// for the father with i2, then the mutation flips.  The parents' words are
// loaded first, so that their latency overlaps the draws.
__global__ void __launch_bounds__(256, 4)   // four CTAs per SM: the grid of four per SM in one wave
k_genomes(const StepConst P, RunState *__restrict__ rs, uint64_t *__restrict__ genome,
          const uint32_t *__restrict__ brec) {
    if (rs->error != 0u) return;
    const uint32_t nbirths = rs->births;
    const uint32_t step = (uint32_t)rs->genome_step;
    const int lane = threadIdx.x & 31;
    const int gw = P.genome_words;
    const int nblk = gw >> 1;
    const uint32_t nbits = (uint32_t)nblk * 64u;
    for (uint32_t g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; g < nbirths;
         g += (gridDim.x * blockDim.x) >> 5) {
        // the record {mother slot, father slot, baby slot, mother ID low, high}
        const uint32_t rv = (lane < 5) ? __ldg(&brec[(size_t)g * 5 + (uint32_t)lane]) : 0u;
        const uint32_t ms = __shfl_sync(FULL_MASK, rv, 0);
        const uint32_t fs = __shfl_sync(FULL_MASK, rv, 1);
        const uint32_t bs = __shfl_sync(FULL_MASK, rv, 2);
        const uint64_t mid = (uint64_t)__shfl_sync(FULL_MASK, rv, 3) | ((uint64_t)__shfl_sync(FULL_MASK, rv, 4) << 32);
        const uint64_t *gm = genome + (size_t)ms * gw;
        const uint64_t *gf = genome + (size_t)fs * gw;
        uint64_t *gb = genome + (size_t)bs * gw;
        // both strands of both parents at the lane's blocks
        uint64_t m0[2] = {0ull, 0ull}, m1[2] = {0ull, 0ull}, f0[2] = {0ull, 0ull}, f1[2] = {0ull, 0ull};
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int b = lane + 32 * h;
            if (b < nblk) {
                m0[h] = gm[b];
                m1[h] = gm[nblk + b];
                f0[h] = gf[b];
                f1[h] = gf[nblk + b];
            }
        }
        const Draw4 d = run_block<false>(P, P.seed, step, (int64_t)mid, kStreamBirth + (uint32_t)lane);
        const int i1 = (int)(birth_draw(d, 1) >> 31);
        const int i2 = (int)(birth_draw(d, 2) >> 31);
        int k = 3, nM = 0, nF = 0;
        if (P.num_crossover == kCrossoverPoisson1) {
            nM = poisson1(birth_draw(d, 3));
            nF = poisson1(birth_draw(d, 4));
            k = 5;
        } else if (P.num_crossover > 0) {
            nM = nF = P.num_crossover;
        }
        const int kMom = k;   // the father's breaks follow the mother's
        k += nM + nF;
        int nmut = 0;
        if (P.has_mutation) {
            const uint32_t u = birth_draw(d, k);
            while (nmut < P.n_binomial && (int64_t)u > P.bino[nmut]) nmut++;
            k++;
        }
        if (k + nmut > kBirthDraws) {
            if (lane == 0) set_error(rs, kErrInternal, 6u);
            continue;
        }
        // the breaks of each parent: those in earlier blocks (their parity
        // picks the strand) and those in the lane's own blocks (the mask)
        BlockMask bmM[2], bmF[2];
        int befM[2] = {0, 0}, befF[2] = {0, 0};
        for (int t = 0; t < nM + nF; t++) {
            const uint32_t pos = (uint32_t)(((uint64_t)nbits * (uint64_t)birth_draw(d, kMom + t)) >> 32);
            const int blk = (int)(pos >> 6);
            const bool mom = t < nM;
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int b = lane + 32 * h;
                if (mom) {
                    befM[h] += (blk < b) ? 1 : 0;
                    if (blk == b) bmM[h].add(pos & 63u);
                } else {
                    befF[h] += (blk < b) ? 1 : 0;
                    if (blk == b) bmF[h].add(pos & 63u);
                }
            }
        }
        uint64_t w0[2], w1[2];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const uint64_t mm = bmM[h].value(), mf = bmF[h].value();
            const bool cm = ((befM[h] & 1) ^ i1) != 0;   // mother: strand taken at the block's start
            const bool cf = ((befF[h] & 1) ^ i2) != 0;
            const uint64_t am = cm ? m1[h] : m0[h], bm = cm ? m0[h] : m1[h];
            const uint64_t af = cf ? f1[h] : f0[h], bf = cf ? f0[h] : f1[h];
            w0[h] = (mm & am) | (~mm & bm);
            w1[h] = (mf & af) | (~mf & bf);
        }
        // BitGeneUtils::mutateNucs (genes/BitGeneUtils.cpp:57-75): flips at
        // wrandi(0, 2 * genome size) over both strands of the newborn
        for (int t = 0; t < nmut; t++) {
            const uint32_t pos = (uint32_t)(((uint64_t)(2u * (uint32_t)P.genome_size) *
                                             (uint64_t)birth_draw(d, k + t)) >> 32);
            const int w = (int)(pos >> 6);
            const uint64_t bit = 1ull << (pos & 63u);
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int b = lane + 32 * h;
                if (w == b) w0[h] ^= bit;
                if (w == nblk + b) w1[h] ^= bit;
            }
        }
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int b = lane + 32 * h;
            if (b < nblk) {
                gb[b] = w0[h];
                gb[nblk + b] = w1[h];
            }
        }
    }
}

// Batches: agents of runs admitted at this step, staged sorted by cell,
// written after the cell's newborns (the cell scan counted them and left
// their first row in ibase).  The last CTA clears the staging count.
__global__ void __launch_bounds__(256)
k_inject(RunState *__restrict__ rs, const BatchBuffers BB, int64_t *__restrict__ id2,
         float *__restrict__ birth2, float *__restrict__ age2, float *__restrict__ lastb2,
         uint8_t *__restrict__ meta2, uint32_t cap) {
    __shared__ uint32_t s_last;
    if (rs->error != 0u) return;
    const uint32_t n = rs->n_staged;
    if (n == 0u) return;
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const uint8_t m = BB.smeta[q];
        if (m == kStagedDead) continue;
        const uint32_t d = BB.scell[q];
        // a countdown of the cell's admitted agents (which leaves it at zero)
        const uint32_t dst = BB.ibase[d] + atomicSub(&BB.inj[d], 1u) - 1u;
        if (dst >= cap) {
            set_error(rs, kErrCapacity, dst);
            continue;
        }
        id2[dst] = BB.sid[q];
        birth2[dst] = BB.sbirth[q];
        age2[dst] = BB.sage[q];
        lastb2[dst] = BB.slastb[q];
        meta2[dst] = m;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = (atomicAdd(BB.inj_ctas_done, 1u) == gridDim.x - 1) ? 1u : 0u;
        if (s_last) {
            *BB.inj_ctas_done = 0u;
            rs->n_staged = 0u;
            __threadfence();
        }
    }
}

// Batches: prepares agents staged as the caller gave them (rows s0..s0+n of
// the staging area, with the state in smeta and the gender in sgender):
// meta byte, cell in the batch's cell space, per-cell counts of the
// admitted agents (inj), the largest ID.  err = {code, info, max ID}.
__global__ void k_batch_stage(uint32_t s0, uint32_t n, uint32_t cell0, uint32_t ncells,
                              const int32_t *__restrict__ cell, uint8_t *__restrict__ smeta,
                              const uint8_t *__restrict__ sgender, const int64_t *__restrict__ sid,
                              uint32_t *__restrict__ scell, uint32_t *__restrict__ inj,
                              unsigned long long *__restrict__ err) {
    long long mx = -1;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t k = base + threadIdx.x;
        bool live = false;
        uint32_t d = 0;
        if (k < n) {
            const uint32_t q = s0 + k;
            const uint8_t st = smeta[q];
            if (st == 0) {
                smeta[q] = kStagedDead;
            } else {
                const int32_t c = cell[k];
                if (c < 0 || (uint32_t)c >= ncells) {
                    atomicCAS(&err[0], 0ull, (unsigned long long)kErrBadCell);
                    smeta[q] = kStagedDead;
                } else {
                    live = true;
                    d = cell0 + (uint32_t)c;
                    scell[q] = d;
                    smeta[q] = (uint8_t)((sgender[q] & 1u) | (st == 5 ? kMetaFertile : 0));
                    mx = max(mx, (long long)sid[q]);
                }
            }
        }
        const uint32_t pos = warp_agg_add(live, d, &inj[live ? d : 0], 1u);
        if (live && pos >= (uint32_t)kMaxCellBig) atomicCAS(&err[0], 0ull, (unsigned long long)kErrCellTooLarge);
    }
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, (long long)__shfl_down_sync(FULL_MASK, mx, o));
    if ((threadIdx.x & 31) == 0 && mx >= 0) atomicMax(reinterpret_cast<long long *>(&err[2]), mx);
}

// ------------------------------------------------------------------ refresh
// After K or the move weights changed between steps (qhg_gpu_set_capacity,
// qhg_gpu_set_move_weights): the current table's per-cell constants, which
// the previous step's cell scan derived from the old values, are derived
// again -- the Verhulst thresholds from the new K and the cell's count, the
// move word from the new cmove -- by the cell's position in the non-empty list.
__global__ void __launch_bounds__(256)
k_refresh_cells(const StepConst P, const BatchRun *__restrict__ runs, const uint32_t *__restrict__ crun,
                const RunState *__restrict__ rs, const uint32_t *__restrict__ nonempty,
                const uint32_t *__restrict__ ne_start, const double *__restrict__ K,
                const uint32_t *__restrict__ cmove, ulonglong2 *__restrict__ vthr, uint32_t *__restrict__ necm,
                uint32_t c0, uint32_t c1) {
    const uint32_t nne = rs->n_nonempty;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nne; i += gridDim.x * blockDim.x) {
        const uint32_t c = nonempty[i];
        if (c < c0 || c >= c1) continue;   // a batch refreshes one run's cells
        if (P.n_verhulst > 0) {
            // a batch's run has its own rates
            const ActionConst &A = runs != nullptr ? runs[crun[c]].act[P.verhulst_act[0]] : P.act[P.verhulst_act[0]];
            vthr[i] = verhulst_thresholds(A, K[c], ne_start[i + 1] - ne_start[i]);
        }
        if (P.has_move) necm[i] = cmove[c];
    }
}

// ------------------------------------------------------------ grid tables
// The grid tables of a run built on the device at qhg_gpu_upload_grid, the
// same as qhg_host_grid_tables / qhg_host_move_tables build on the host
// (which serve the batch form and the updates between steps): per cell the
// reverse slots (3 bits per neighbour slot: the cell's slot in the
// neighbour's list), the move word (neighbour count, slots holding a
// neighbour, slots a WeightedMove may enter) and SingleEvaluator's own
// weight (actions/SingleEvaluator.cpp:174-241); then the cumulative weights
// and WeightedMove's integer thresholds.  A cell that fails records
// (cell << 8 | problem) in *bad (the smallest wins): 1 more than 6
// neighbours, 2 a neighbour index out of range, 3 a link without its
// reverse, 4 a total weight not positive and finite, 5 a weight not finite.
__global__ void __launch_bounds__(256)
k_grid_cells(int C, const int32_t *__restrict__ nbr6, const uint8_t *__restrict__ nnbr,
             const double *__restrict__ K, int wm, uint32_t *__restrict__ rev, uint32_t *__restrict__ cmove,
             double *__restrict__ W, unsigned long long *__restrict__ bad) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < C; c += gridDim.x * blockDim.x) {
        const int nn = nnbr[c];
        uint32_t why = nn > 6 ? 1u : 0u, rv = 0u, vm = 0u;
        for (int j = 0; j < 6 && why == 0u; j++) {
            const int d = nbr6[(size_t)c * 6 + j];
            if (d >= C || d < -1) {
                why = 2u;
                break;
            }
            if (d >= 0) vm |= 1u << j;
            if (j >= nn || d < 0) continue;
            int k = -1;
            for (int q = 0; q < (int)nnbr[d] && q < 6; q++) {
                if (nbr6[(size_t)d * 6 + q] == c) {
                    k = q;
                    break;
                }
            }
            if (k < 0) why = 3u;
            else rv |= (uint32_t)k << (3 * j);
        }
        if (why != 0u) {
            atomicMin(bad, ((unsigned long long)c << 8) | why);
            continue;
        }
        rev[c] = rv;
        // no ice at the upload: every slot holding a neighbour may be entered
        cmove[c] = (uint32_t)nn | (vm << 8) | (vm << 24);
        if (wm) W[(size_t)c * 7] = K[c] > 0.0 ? K[c] : 0.0;
    }
}

__global__ void __launch_bounds__(256)
k_grid_weights(int C, const int32_t *__restrict__ nbr6, const uint8_t *__restrict__ nnbr, double *__restrict__ W,
               uint64_t *__restrict__ wthr, uint32_t *__restrict__ cmove, unsigned long long *__restrict__ bad) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < C; c += gridDim.x * blockDim.x) {
        // cumulative weights: W[c][i+1] = W[c][i] + max(0, neighbour i's own weight)
        double row[7];
        row[0] = W[(size_t)c * 7];
        double dW = row[0];
        for (int i = 0; i < 6; i++) {
            const int ni = nbr6[(size_t)c * 6 + i];
            double dCW = ni >= 0 ? W[(size_t)ni * 7] : 0.0;
            dCW = dCW > 0.0 ? dCW : 0.0;
            dW = __dadd_rn(dW, dCW);
            row[i + 1] = dW;
        }
        for (int i = 1; i < 7; i++) W[(size_t)c * 7 + i] = row[i];
        // thresholds: the smallest draw u with wrandd() * W[n] >= W[j]
        // (u / 2^32 is exact, so it is u * 2^-32), as a running maximum
        const int nn = nnbr[c];
        const double Wn = row[nn];
        uint32_t cm = cmove[c] & ~(1u << 16);
        uint64_t *wt = wthr + (size_t)c * 6;
        if (row[0] == Wn) {
            cm |= 1u << 16;
            for (int j = 0; j < 6; j++) wt[j] = 0ull;
        } else if (!(Wn > 0.0) || !isfinite(Wn)) {
            atomicMin(bad, ((unsigned long long)c << 8) | 4u);
        } else {
            const double guess = __ddiv_rn(4294967296.0, Wn);   // where the search starts
            uint64_t run = 0ull;
            bool ok = true;
            for (int j = 0; j < nn; j++) {
                const double x = row[j];
                if (!isfinite(x)) {
                    ok = false;
                    break;
                }
                const double g = floor(__dmul_rn(x, guess));
                uint64_t u = (g <= 0.0) ? 0ull : (g >= 4294967296.0 ? 4294967296ull : (uint64_t)g);
                while (u > 0ull && __dmul_rn((double)(u - 1ull) * 0x1p-32, Wn) >= x) u--;
                while (u < 4294967296ull && __dmul_rn((double)u * 0x1p-32, Wn) < x) u++;
                run = max(run, u);
                wt[j] = run;
            }
            if (!ok) atomicMin(bad, ((unsigned long long)c << 8) | 5u);
            for (int j = nn; j < 6; j++) wt[j] = 4294967296ull;
        }
        cmove[c] = cm;
    }
}

// ------------------------------------------------------------------ upload
// An upload on the device: the caller's columns are copied as they are into
// staging buffers; k_upload_count counts the live agents of each cell (into
// the class-count slot 0 of the cell, as if they all stayed), k_cell_scan
// lays out the table from those counts exactly as after a step (first rows,
// non-empty cells, tiles, Verhulst thresholds), and k_upload_place puts each
// agent at its cell's first row + a countdown of the cell's count (which
// leaves the counts at zero, as a step's scatter does).  The order of the
// agents within a cell is arbitrary: nothing depends on it.
__global__ void k_upload_count(RunState *__restrict__ rs, const int32_t *__restrict__ cell,
                               const uint8_t *__restrict__ state, const int64_t *__restrict__ id, int64_t n,
                               int C, uint32_t *__restrict__ clsc) {
    long long mx = -1;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t q = base + threadIdx.x;
        bool live = false;
        int32_t c = 0;
        if (q < n && state[q] != 0) {
            c = cell[q];
            if (c < 0 || c >= C) set_error(rs, kErrBadCell, (uint32_t)q);
            else live = true;
            mx = max(mx, (long long)id[q]);
        }
        warp_agg_add(live, live ? (uint32_t)c : 0u, &clsc[(size_t)(live ? c : 0) * kCls], 1u);
    }
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, (long long)__shfl_down_sync(FULL_MASK, mx, o));
    if ((threadIdx.x & 31) == 0 && mx >= 0) atomicMax(reinterpret_cast<long long *>(&rs->next_id), mx);
}

__global__ void k_upload_place(RunState *__restrict__ rs, const int32_t *__restrict__ cell,
                               const uint8_t *__restrict__ gender, const uint8_t *__restrict__ state,
                               const int64_t *__restrict__ sid, const float *__restrict__ sbirth,
                               const float *__restrict__ sage, const float *__restrict__ slastb, int64_t n,
                               uint32_t cap, const uint32_t *__restrict__ sbase, uint32_t *__restrict__ clsc,
                               int64_t *__restrict__ id, float *__restrict__ birth, float *__restrict__ age,
                               float *__restrict__ lastb, uint8_t *__restrict__ meta, int32_t *__restrict__ gslot) {
    if (rs->error != 0u) return;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const uint8_t st = state[q];
        if (st == 0) continue;
        const int32_t c = cell[q];
        const uint32_t pos = sbase[c] + atomicSub(&clsc[(size_t)c * kCls], 1u) - 1u;
        if (pos >= cap) {
            set_error(rs, kErrCapacity, pos);
            continue;
        }
        id[pos] = sid[q];
        birth[pos] = sbirth[q];
        age[pos] = sage[q];
        lastb[pos] = slastb[q];
        meta[pos] = (uint8_t)((gender[q] & 1u) | (st == 5 ? kMetaFertile : 0));
        if (gslot) gslot[pos] = (int32_t)q;   // genome slot = input row
    }
}

// genomes of the table's rows in row order (download)
__global__ void k_gather_genomes(const int32_t *__restrict__ gslot, const uint64_t *__restrict__ genome,
                                 uint32_t n, int words, uint32_t slots, uint64_t *__restrict__ out) {
    const uint64_t total = (uint64_t)n * (uint64_t)words;
    for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total;
         q += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t row = (uint32_t)(q / (uint64_t)words);
        const int w = (int)(q % (uint64_t)words);
        const int32_t sl = gslot[row];
        out[q] = (sl >= 0 && (uint32_t)sl < slots) ? genome[(size_t)sl * words + w] : 0ull;
    }
}

// the download's per-row columns of a single run's table, built on the
// device: the cell of each row (one warp per non-empty cell), the gender and
// the life state from the meta byte, and -- where the table's ages are
// derived -- the ages (float)(step - 1) - birth, written into the table's
// own age column
__global__ void k_download_cols(const uint32_t *__restrict__ nonempty, const uint32_t *__restrict__ ne_start,
                                uint32_t nne, uint32_t n, const uint8_t *__restrict__ meta,
                                const float *__restrict__ birth, float t_prev, int derived,
                                int32_t *__restrict__ cell_out, uint8_t *__restrict__ gender_out,
                                uint8_t *__restrict__ state_out, float *__restrict__ age) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < nne; k += warps) {
        const int32_t c = (int32_t)nonempty[k];
        const uint32_t a = ne_start[k], b = ne_start[k + 1];
        for (uint32_t i = a + lane; i < b && i < n; i += 32u) cell_out[i] = c;
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint8_t m = meta[i];
        gender_out[i] = m & kMetaGender;
        state_out[i] = (m & kMetaFertile) ? QHG_LS_FERTILE_DEV : QHG_LS_ALIVE_DEV;
        if (derived) age[i] = __fsub_rn(t_prev, birth[i]);
    }
}

// rows of one batch run in the current table: the cell of each row and the
// agents per cell (either output may be null)
__global__ void k_run_cells(const uint32_t *__restrict__ nonempty, const uint32_t *__restrict__ ne_start,
                            uint32_t nne, uint32_t cell0, uint32_t cell1, uint32_t row0, uint32_t nrows,
                            uint32_t *__restrict__ row_cell, uint32_t *__restrict__ counts) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nne; k += gridDim.x * blockDim.x) {
        const uint32_t c = nonempty[k];
        if (c < cell0 || c >= cell1) continue;
        const uint32_t r0 = ne_start[k], r1 = ne_start[k + 1];
        if (counts) counts[c - cell0] = r1 - r0;
        if (row_cell) {
            for (uint32_t r = r0; r < r1; r++) {
                if (r >= row0 && r - row0 < nrows) row_cell[r - row0] = c;
            }
        }
    }
}

}  // namespace qhg

extern "C" int qhg_launch_refresh_cells(const qhg::StepConst *P, const qhg::RunState *rs, const uint32_t *nonempty,
                                        const uint32_t *ne_start, const double *K, const uint32_t *cmove,
                                        ulonglong2 *vthr, uint32_t *necm, int grid, cudaStream_t stream) {
    qhg::k_refresh_cells<<<std::max(1, grid), 256, 0, stream>>>(*P, nullptr, nullptr, rs, nonempty, ne_start, K, cmove,
                                                                 vthr, necm, 0u, 0xffffffffu);
    return (int)cudaGetLastError();
}

extern "C" int qhg_launch_ms_fill(uint32_t c0, uint32_t c1, int mode, const uint32_t *origin, uint32_t norigin,
                                  int32_t *hops, double *dist, double *time, int32_t *chops,
                                  unsigned long long *cdist, unsigned long long *ckey, double *D, cudaStream_t stream) {
    if (c1 > c0) {
        const uint32_t g = std::min<uint32_t>((c1 - c0 + 255u) / 256u, 4096u);
        qhg::k_ms_fill<<<g, 256, 0, stream>>>(c0, c1, mode, hops, dist, time, chops, cdist, ckey, D);
    }
    if (norigin > 0u) {
        const uint32_t g = std::min<uint32_t>((norigin + 255u) / 256u, 4096u);
        qhg::k_ms_origins<<<g, 256, 0, stream>>>(c0, c1, origin, norigin, hops, dist, time);
    }
    return (int)cudaGetLastError();
}

extern "C" int qhg_launch_grid_tables(int C, const int32_t *nbr6, const uint8_t *nnbr, const double *K, int wm,
                                      uint32_t *rev, uint32_t *cmove, double *W, uint64_t *wthr,
                                      unsigned long long *bad, int pass, cudaStream_t stream) {
    const int g = std::max(1, std::min((C + 255) / 256, 152 * 16));
    if (pass == 0) qhg::k_grid_cells<<<g, 256, 0, stream>>>(C, nbr6, nnbr, K, wm, rev, cmove, W, bad);
    else qhg::k_grid_weights<<<g, 256, 0, stream>>>(C, nbr6, nnbr, W, wthr, cmove, bad);
    return (int)cudaGetLastError();
}

extern "C" int qhg_launch_refresh_cells_batch(const qhg::StepConst *P, const qhg::BatchRun *runs, const uint32_t *crun,
                                              const qhg::RunState *rs, const uint32_t *nonempty,
                                              const uint32_t *ne_start, const double *K, const uint32_t *cmove,
                                              ulonglong2 *vthr, uint32_t *necm, uint32_t cell0, uint32_t cell1,
                                              int grid, cudaStream_t stream) {
    qhg::k_refresh_cells<<<std::max(1, grid), 256, 0, stream>>>(*P, runs, crun, rs, nonempty, ne_start, K, cmove, vthr,
                                                                 necm, cell0, cell1);
    return (int)cudaGetLastError();
}


extern "C" int qhg_launch_run_cells(const uint32_t *nonempty, const uint32_t *ne_start, uint32_t n_nonempty,
                                    uint32_t cell0, uint32_t cell1, uint32_t row0, uint32_t nrows,
                                    uint32_t *row_cell, uint32_t *counts, cudaStream_t stream) {
    const uint32_t blocks = std::min<uint32_t>((n_nonempty + 255) / 256, 4096u);
    if (blocks > 0) {
        qhg::k_run_cells<<<blocks, 256, 0, stream>>>(nonempty, ne_start, n_nonempty, cell0, cell1, row0, nrows,
                                                     row_cell, counts);
    }
    return (int)cudaGetLastError();
}

extern "C" int qhg_launch_batch_stage(uint32_t s0, uint32_t n, uint32_t cell0, uint32_t ncells, const int32_t *cell,
                                      uint8_t *smeta, const uint8_t *sgender, const int64_t *sid, uint32_t *scell,
                                      uint32_t *inj, unsigned long long *err, cudaStream_t stream) {
    const uint32_t blk = std::min<uint32_t>((n + 255) / 256, 65535u);
    if (blk > 0) {
        qhg::k_batch_stage<<<blk, 256, 0, stream>>>(s0, n, cell0, ncells, cell, smeta, sgender, sid, scell, inj, err);
    }
    return (int)cudaGetLastError();
}

extern "C" int qhg_launch_upload(const qhg::StepConst *P, qhg::RunState *rs, const qhg::StepBuffers *B,
                                 const int32_t *cell, const uint8_t *gender, const uint8_t *state, const int64_t *sid,
                                 const float *sbirth, const float *sage, const float *slastb, int64_t n,
                                 int32_t *gslot_out, cudaStream_t stream) {
    using namespace qhg;
    const int sitems = scan_items(P->num_cells);
    const int ntiles = (P->num_cells + kScanThreads * sitems - 1) / (kScanThreads * sitems);
    const int64_t blk = std::min<int64_t>((n + 255) / 256, 65535);
    if (n > 0) {
        k_upload_count<<<(unsigned)blk, 256, 0, stream>>>(rs, cell, state, sid, n, P->num_cells, B->clsc);
    }
    BatchBuffers BB;
    memset(&BB, 0, sizeof(BB));
    if (sitems == 2) {
        k_cell_scan<false, 2><<<ntiles, kScanThreads, 0, stream>>>(
            *P, BB, rs, B->nbr, B->nnbr, B->rev, B->clsc, B->K, B->vthr2, B->cmove, B->necm2, B->sbase, B->bbase,
            B->bidbase, B->obase, B->nonempty2, B->ne_start2, B->tile_first2, B->tile_flag, B->tile_agg, B->tile_incl);
    } else {
        k_cell_scan<false, 1><<<ntiles, kScanThreads, 0, stream>>>(
            *P, BB, rs, B->nbr, B->nnbr, B->rev, B->clsc, B->K, B->vthr2, B->cmove, B->necm2, B->sbase, B->bbase,
            B->bidbase, B->obase, B->nonempty2, B->ne_start2, B->tile_first2, B->tile_flag, B->tile_agg, B->tile_incl);
    }
    if (n > 0) {
        k_upload_place<<<(unsigned)blk, 256, 0, stream>>>(rs, cell, gender, state, sid, sbirth, sage, slastb, n,
                                                        P->capacity, B->sbase, B->clsc, B->id2, B->birth2,
                                                        B->age2, B->lastb2, B->meta2, gslot_out);
    }
    return (int)cudaGetLastError();
}

extern "C" int qhg_launch_occupancy(const qhg::RunState *rs, const uint32_t *nonempty, int32_t *occ, int grid,
                                    cudaStream_t stream) {
    qhg::k_occupancy<<<std::max(1, grid), 256, 0, stream>>>(rs, nonempty, occ, nullptr, nullptr);
    return (int)cudaGetLastError();
}

extern "C" int qhg_launch_download_cols(const uint32_t *nonempty, const uint32_t *ne_start, uint32_t nne, uint32_t n,
                                        const uint8_t *meta, const float *birth, float t_prev, int derived,
                                        int32_t *cell_out, uint8_t *gender_out, uint8_t *state_out, float *age,
                                        cudaStream_t stream) {
    const uint32_t work = std::max(nne * 32u, n);
    const unsigned blocks = (unsigned)std::max<uint32_t>(1u, std::min<uint32_t>((work + 255u) / 256u, 152u * 16u));
    qhg::k_download_cols<<<blocks, 256, 0, stream>>>(nonempty, ne_start, nne, n, meta, birth, t_prev, derived,
                                                      cell_out, gender_out, state_out, age);
    return (int)cudaGetLastError();
}

extern "C" int qhg_launch_gather_genomes(const int32_t *gslot, const uint64_t *genome, uint32_t n, int words,
                                         uint32_t slots, uint64_t *out, cudaStream_t stream) {
    const uint64_t total = (uint64_t)n * (uint64_t)words;
    const uint64_t blocks = std::min<uint64_t>((total + 255) / 256, 65535);
    if (blocks > 0) qhg::k_gather_genomes<<<(unsigned)blocks, 256, 0, stream>>>(gslot, genome, n, words, slots, out);
    return (int)cudaGetLastError();
}

// dynamic shared memory of the tile kernels (above the 48 KB default: the
// attribute is set once per device before the first launch)
template <int PROG, bool BATCH, bool BIG>
static void set_actions_attr() {
    cudaFuncSetAttribute(qhg::k_actions<PROG, BATCH, BIG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sizeof(qhg::ActionsSmemT<qhg::Tile<BIG>::kMax, qhg::Tile<BIG>::kThreads, BATCH>));
}
template <bool BATCH, bool BIG>
static void set_scatter_attr() {
    cudaFuncSetAttribute(qhg::k_scatter<BATCH, BIG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sizeof(qhg::ScatterSmemT<qhg::Tile<BIG>::kMax, qhg::Tile<BIG>::kThreads>));
}

template <bool BATCH>
static void set_scatter_cell_attr() {
    cudaFuncSetAttribute(qhg::k_scatter_cell<BATCH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(2 * qhg::kCellWarps * qhg::scatter_stage_bytes(true, true)));
}

template <int PROG, bool BATCH>
static void set_cell_attr() {
    cudaFuncSetAttribute(qhg::k_actions_cell<PROG, BATCH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(sizeof(qhg::CellWarpSmem) * qhg::kCellWarps));
}

static void set_tile_attributes() {
    static bool done[64] = {false};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64 || done[dev]) return;
    set_cell_attr<0, false>(); set_cell_attr<1, false>(); set_cell_attr<2, false>(); set_cell_attr<3, false>();
    set_cell_attr<0, true>(); set_cell_attr<1, true>();
    set_scatter_cell_attr<false>(); set_scatter_cell_attr<true>();
    set_actions_attr<0, false, false>(); set_actions_attr<1, false, false>();
    set_actions_attr<2, false, false>(); set_actions_attr<3, false, false>();
    set_actions_attr<0, true, false>(); set_actions_attr<1, true, false>();
    set_actions_attr<0, false, true>(); set_actions_attr<0, true, true>();
    set_scatter_attr<false, false>(); set_scatter_attr<true, false>();
    set_scatter_attr<false, true>(); set_scatter_attr<true, true>();
    done[dev] = true;
}

// grids of the cell form: every SM filled with as many CTAs of each cell
// kernel as fit (once per device)
struct CellGrids {
    int actions, actions0;   // action kernel: specialised programs, the interpreter
    // scatter [batch]: as many CTAs as fit with the largest staging buffers
    // (age and genome-slot columns), three per SM.  Grids sized for the
    // run's own buffers (four or five CTAs, 64 or 48 registers) measured
    // slower on the 20M-agent run (0.23 / 0.27 ms against 0.20 ms), though
    // four were 5 % faster on an 8M-agent one
    int scatter[2];
};
static CellGrids cell_grids() {
    static CellGrids g[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) dev = 0;
    if (g[dev].actions == 0) {
        int nsm = 1, a = 0, a0 = 0;
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, qhg::k_actions_cell<2, false>, qhg::kCellThreads,
                                                      sizeof(qhg::CellWarpSmem) * qhg::kCellWarps);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a0, qhg::k_actions_cell<0, false>, qhg::kCellThreads,
                                                      sizeof(qhg::CellWarpSmem) * qhg::kCellWarps);
        g[dev].actions = std::max(1, nsm) * std::max(1, a);
        g[dev].actions0 = std::max(1, nsm) * std::max(1, a0);
        const size_t sm = 2 * qhg::kCellWarps * qhg::scatter_stage_bytes(true, true);
        int b = 0, bb = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, qhg::k_scatter_cell<false>, qhg::kCellThreads, sm);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bb, qhg::k_scatter_cell<true>, qhg::kCellThreads, sm);
        g[dev].scatter[0] = std::max(1, nsm) * std::max(1, b);
        g[dev].scatter[1] = std::max(1, nsm) * std::max(1, bb);
    }
    return g[dev];
}

// One step's launches come in four phases: the action kernels, the
// MoveStats candidates and the cell scan, the scatters, the work after the
// commit.  The action kernel and the scatter exist in three forms; `form`
// selects one (kFormTile, kFormBig, kFormCell) or, with -1, launches all of
// them, and those that do not match the step's table (RunState::form, set by
// the previous step) return at once.  Steps launch all forms: graphs whose
// switch nodes launch only the step's form measured slower on GB300 (the
// large run's step +3 %, steps of small runs markedly slower) than the three
// early-returning launches they save.
struct StepLaunch {
    const qhg::StepConst *P;
    qhg::RunState *rs;
    const qhg::StepBuffers *B;
    qhg::BatchBuffers BB;
    bool batch;
    qhg::LaunchShape L;
    cudaStream_t stream;
};

static StepLaunch step_launch(const qhg::StepConst *P, qhg::RunState *rs, const qhg::StepBuffers *B,
                              const qhg::BatchBuffers *BBp, const qhg::LaunchShape &L, cudaStream_t stream) {
    StepLaunch S;
    S.P = P; S.rs = rs; S.B = B; S.batch = BBp != nullptr; S.L = L; S.stream = stream;
    if (S.batch) S.BB = *BBp;
    else memset(&S.BB, 0, sizeof(S.BB));
    return S;
}

static void launch_actions(const StepLaunch &S, int form) {
    using namespace qhg;
    const StepConst *P = S.P;
    RunState *rs = S.rs;
    const StepBuffers *B = S.B;
    const BatchBuffers &BB = S.BB;
    const LaunchShape &L = S.L;
    cudaStream_t stream = S.stream;
    const bool batch = S.batch;
    constexpr size_t kSmC = sizeof(CellWarpSmem) * kCellWarps;
    const CellGrids CG = cell_grids();
    const size_t kSmA = batch ? sizeof(ActionsSmemT<Tile<false>::kMax, Tile<false>::kThreads, true>)
                              : sizeof(ActionsSmemT<Tile<false>::kMax, Tile<false>::kThreads, false>);
    const size_t kSmAB = batch ? sizeof(ActionsSmemT<Tile<true>::kMax, Tile<true>::kThreads, true>)
                               : sizeof(ActionsSmemT<Tile<true>::kMax, Tile<true>::kThreads, false>);
    const bool tile = form < 0 || form == (int)kFormTile, cell = form < 0 || form == (int)kFormCell;
    const bool big = form < 0 || form == (int)kFormBig;
#define QHG_LAUNCH_ACTIONS(PR, BT, BG, GRID, SM)                                                          \
    k_actions<PR, BT, BG><<<GRID, Tile<BG>::kThreads, SM, stream>>>(                                      \
        *P, BB, rs, B->nonempty, B->ne_start, B->tile_first, B->id, B->birth, B->age, B->lastb, B->meta, \
        B->vthr, B->wthr, B->necm, B->outc, B->father, B->brank, B->clsc)
#define QHG_LAUNCH_CELL(PR, BT)                                                                            \
    k_actions_cell<PR, BT><<<(PR > 0 ? CG.actions : CG.actions0), kCellThreads, kSmC, stream>>>(            \
        *P, BB, rs, B->nonempty, B->ne_start, B->id, B->birth, B->age, B->lastb, B->meta, B->vthr, B->wthr, \
        B->necm, B->outc, B->father, B->clsc)
#define QHG_FORMS(PR, BT)                                                      \
    do {                                                                       \
        if (tile) QHG_LAUNCH_ACTIONS(PR, BT, false, L.actions_grid, kSmA);     \
        if (cell) QHG_LAUNCH_CELL(PR, BT);                                     \
    } while (0)
    if (batch) {
        switch (P->program) {
        case 1: QHG_FORMS(1, true); break;
        default: QHG_FORMS(0, true); break;
        }
        if (big) QHG_LAUNCH_ACTIONS(0, true, true, L.big_grid, kSmAB);
    } else {
        switch (P->program) {
        case 1: QHG_FORMS(1, false); break;
        case 2: QHG_FORMS(2, false); break;
        case 3: QHG_FORMS(3, false); break;
        default: QHG_FORMS(0, false); break;
        }
        if (big) QHG_LAUNCH_ACTIONS(0, false, true, L.big_grid, kSmAB);
    }
#undef QHG_FORMS
#undef QHG_LAUNCH_CELL
#undef QHG_LAUNCH_ACTIONS
}

static void launch_scan(const StepLaunch &S) {
    using namespace qhg;
    const StepConst *P = S.P;
    RunState *rs = S.rs;
    const StepBuffers *B = S.B;
    const BatchBuffers &BB = S.BB;
    cudaStream_t stream = S.stream;
    const bool batch = S.batch;
    const int sitems = S.L.scan_items > 0 ? std::min(S.L.scan_items, 2) : scan_items(P->num_cells);
    const int ntiles = (P->num_cells + kScanThreads * sitems - 1) / (kScanThreads * sitems);
    const int ms_grid = std::max(1, std::min((P->num_cells + 7) / 8, 152 * 16));
    if (B->ms_mode >= 0) {
#define QHG_LAUNCH_MS_PICK(MD, PS)                                                                          \
    k_ms_pick<MD, PS><<<ms_grid, 256, 0, stream>>>(rs, B->nonempty, B->ne_start, B->id, B->outc, B->nbr, B->ms_D, \
                                                  B->ms_hops, B->ms_dist, B->ms_chops, B->ms_cdist, B->ms_ckey)
        switch (B->ms_mode) {
        case kMsFirst: QHG_LAUNCH_MS_PICK(kMsFirst, 0); QHG_LAUNCH_MS_PICK(kMsFirst, 1); break;
        case kMsMin: QHG_LAUNCH_MS_PICK(kMsMin, 0); break;
        default: QHG_LAUNCH_MS_PICK(kMsLast, 0); QHG_LAUNCH_MS_PICK(kMsLast, 1); break;
        }
#undef QHG_LAUNCH_MS_PICK
    }
#define QHG_LAUNCH_SCAN(BT, IT)                                                                             \
    k_cell_scan<BT, IT><<<ntiles, kScanThreads, 0, stream>>>(                                               \
        *P, BB, rs, B->nbr, B->nnbr, B->rev, B->clsc, B->K, B->vthr2, B->cmove, B->necm2, B->sbase, B->bbase, B->bidbase,       \
        B->obase, B->nonempty2, B->ne_start2, B->tile_first2, B->tile_flag, B->tile_agg, B->tile_incl)
    if (batch) {
        if (sitems == 2) QHG_LAUNCH_SCAN(true, 2);
        else QHG_LAUNCH_SCAN(true, 1);
    } else {
        if (sitems == 2) QHG_LAUNCH_SCAN(false, 2);
        else QHG_LAUNCH_SCAN(false, 1);
    }
#undef QHG_LAUNCH_SCAN
}

static void launch_scatter(const StepLaunch &S, int form) {
    using namespace qhg;
    const StepConst *P = S.P;
    RunState *rs = S.rs;
    const StepBuffers *B = S.B;
    const BatchBuffers &BB = S.BB;
    const LaunchShape &L = S.L;
    cudaStream_t stream = S.stream;
    const bool batch = S.batch;
    const CellGrids CG = cell_grids();
    const size_t kSmSC = (size_t)2 * kCellWarps * scatter_stage_bytes(!P->age_from_birth, P->genome_words > 0);
    constexpr size_t kSmS = sizeof(ScatterSmemT<Tile<false>::kMax, Tile<false>::kThreads>);
    constexpr size_t kSmSB = sizeof(ScatterSmemT<Tile<true>::kMax, Tile<true>::kThreads>);
    const bool tile = form < 0 || form == (int)kFormTile, cell = form < 0 || form == (int)kFormCell;
    const bool big = form < 0 || form == (int)kFormBig;
#define QHG_LAUNCH_SCATTER(BT, BG, GRID, SM)                                                                \
    k_scatter<BT, BG><<<GRID, Tile<BG>::kThreads, SM, stream>>>(                                            \
        *P, BB, rs, B->nonempty, B->ne_start, B->tile_first, B->id, B->birth, B->age, B->lastb, B->outc,   \
        B->father, B->brank, B->nnbr, B->sbase, B->bbase, B->bidbase, B->obase, B->clsc, B->id2, B->birth2, \
        B->age2, B->lastb2, B->meta2, B->blog, B->blog_cap, B->gslot, B->gslot2, B->freelist,              \
        B->freelist2, B->brec)
#define QHG_LAUNCH_SCATTER_CELL(BT)                                                                        \
    k_scatter_cell<BT><<<CG.scatter[BT ? 1 : 0], kCellThreads, kSmSC, stream>>>(                             \
        *P, BB, rs, B->nonempty, B->ne_start, B->id, B->birth, B->age, B->lastb, B->outc, B->father,       \
        B->sbase, B->bbase, B->bidbase, B->obase, B->clsc, B->id2, B->birth2, B->age2, B->lastb2,          \
        B->meta2, B->blog, B->blog_cap, B->gslot, B->gslot2, B->freelist, B->freelist2, B->brec)
    if (batch) {
        if (tile) QHG_LAUNCH_SCATTER(true, false, L.scatter_grid, kSmS);
        if (cell) QHG_LAUNCH_SCATTER_CELL(true);
        if (big) QHG_LAUNCH_SCATTER(true, true, L.big_grid, kSmSB);
    } else {
        if (tile) QHG_LAUNCH_SCATTER(false, false, L.scatter_grid, kSmS);
        if (cell) QHG_LAUNCH_SCATTER_CELL(false);
        if (big) QHG_LAUNCH_SCATTER(false, true, L.big_grid, kSmSB);
    }
#undef QHG_LAUNCH_SCATTER_CELL
#undef QHG_LAUNCH_SCATTER
}

static void launch_post(const StepLaunch &S, cudaEvent_t *ev) {
    using namespace qhg;
    const StepConst *P = S.P;
    RunState *rs = S.rs;
    const StepBuffers *B = S.B;
    const BatchBuffers &BB = S.BB;
    const LaunchShape &L = S.L;
    cudaStream_t stream = S.stream;
    const bool batch = S.batch;
    if (B->occ != nullptr) {
        k_occupancy<<<std::max(1, L.scatter_grid), 256, 0, stream>>>(rs, B->nonempty2, B->occ,
                                                                      batch ? BB.runs : nullptr,
                                                                      batch ? BB.crun : nullptr);
    }
    if (B->ms_mode >= 0) {
        const int mg = std::max(1, std::min((P->num_cells + 255) / 256, 152 * 8));
#define QHG_LAUNCH_MS_MERGE(MD)                                                                             \
    k_ms_merge<MD><<<mg, 256, 0, stream>>>(rs, P->num_cells, B->ms_hops, B->ms_dist, B->ms_time, B->ms_chops, \
                                           B->ms_cdist, B->ms_ckey, batch ? BB.runs : nullptr,             \
                                           batch ? BB.crun : nullptr)
        switch (B->ms_mode) {
        case kMsFirst: QHG_LAUNCH_MS_MERGE(kMsFirst); break;
        case kMsMin: QHG_LAUNCH_MS_MERGE(kMsMin); break;
        default: QHG_LAUNCH_MS_MERGE(kMsLast); break;
        }
#undef QHG_LAUNCH_MS_MERGE
    }
    if (batch) {
        k_inject<<<L.scatter_grid, 256, 0, stream>>>(rs, BB, B->id2, B->birth2, B->age2, B->lastb2, B->meta2,
                                                     P->capacity);
        if (ev) cudaEventRecord(ev[4], stream);
    } else if (P->genome_words > 0) {
        k_genomes<<<L.scatter_grid, 256, 0, stream>>>(*P, rs, B->genome, B->brec);
        if (ev) cudaEventRecord(ev[4], stream);
    }
}

static void launch_kernels(const qhg::StepConst *P, qhg::RunState *rs, const qhg::StepBuffers *B,
                           const qhg::BatchBuffers *BBp, const qhg::LaunchShape &L, cudaStream_t stream,
                           cudaEvent_t *ev) {
    set_tile_attributes();
    const StepLaunch S = step_launch(P, rs, B, BBp, L, stream);
    if (ev) cudaEventRecord(ev[0], stream);
    launch_actions(S, -1);
    if (ev) cudaEventRecord(ev[1], stream);
    launch_scan(S);
    if (ev) cudaEventRecord(ev[2], stream);
    launch_scatter(S, -1);
    if (ev) cudaEventRecord(ev[3], stream);
    launch_post(S, ev);
}

extern "C" int qhg_launch_step(const qhg::StepConst *P, qhg::RunState *rs, const qhg::StepBuffers *B,
                               const qhg::BatchBuffers *BB, const qhg::LaunchShape *L, cudaStream_t stream) {
    launch_kernels(P, rs, B, BB, *L, stream, nullptr);
    return (int)cudaGetLastError();
}

extern "C" int qhg_launch_step_timed(const qhg::StepConst *P, qhg::RunState *rs, const qhg::StepBuffers *B,
                                     const qhg::BatchBuffers *BB, const qhg::LaunchShape *L, cudaStream_t stream,
                                     cudaEvent_t *ev) {
    launch_kernels(P, rs, B, BB, *L, stream, ev);
    return (int)cudaGetLastError();
}

// CTAs of each tile kernel (normal form) that fit on one SM at once
// (the launch shape of the tile form; the cell form sizes its grids itself)
extern "C" void qhg_tile_ctas_per_sm(int *actions, int *scatter) {
    int a = 0, b = 0;
    set_tile_attributes();
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &a, qhg::k_actions<0, false, false>, qhg::kTileThreads,
        sizeof(qhg::ActionsSmemT<qhg::Tile<false>::kMax, qhg::Tile<false>::kThreads, false>));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &b, qhg::k_scatter<false, false>, qhg::kTileThreads,
        sizeof(qhg::ScatterSmemT<qhg::Tile<false>::kMax, qhg::Tile<false>::kThreads>));
    *actions = a > 0 ? a : 1;
    *scatter = b > 0 ? b : 1;
}

// first draw of action a of specialised program p (the host checks its windows against it)
extern "C" uint32_t qhg_program_window(int p, int a) { return qhg::prog_window(p, a); }

// the specialised action program matching a run's action list, 0 if none
extern "C" int qhg_match_program(const int32_t *types, int n) {
    for (int p = 1; p < qhg::kNumPrograms; p++) {
        if (qhg::prog_len(p) != n) continue;
        bool ok = true;
        for (int a = 0; a < n && ok; a++) ok = (qhg::prog_act(p, a) == types[a]);
        if (ok) return p;
    }
    return 0;
}
