// Device-side definitions shared by the kernels and the host API of
// libqhg_gpu.so: the Philox4x32-10 generator, the per-run state kept in
// device memory, and the per-step constants passed to every kernel.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace qhg {

// ---------------------------------------------------------------- layout
constexpr int kMaxActions = 16;
constexpr int kMaxVerhulst = 1;          // Verhulst / VerhulstVarK actions per population
constexpr int kMaxCell = 512;            // agents per cell of the normal tile kernels
constexpr int kMaxCellBig = 4608;        // agents one cell may hold (big-cell tile kernels)
// agent kernels work on cell-aligned tiles: tile t holds the non-empty cells
// whose first row lies in [t*kTileAgents, (t+1)*kTileAgents)
constexpr int kTileAgents = 512;
constexpr int kTileMax = kTileAgents + kMaxCell;  // rows a tile can hold
constexpr int kTileCells = kTileAgents;           // cells a tile can hold
constexpr int kTileThreads = 256;
// geometry of the tile kernels: the normal form (256 threads, cells of up to
// kMaxCell agents) and the big-cell form used for steps in which some cell
// holds more (1024 threads, one CTA per SM)
template <bool BIG>
struct Tile {
    static constexpr int kThreads = BIG ? 1024 : kTileThreads;
    static constexpr int kMax = BIG ? kTileAgents + kMaxCellBig : kTileMax;
};
// The kernels of a step, chosen from the table the step reads: cell-aligned
// tiles of kTileAgents agents for tables of small cells, one warp per cell
// for tables whose non-empty cells hold kDenseCell agents or more on average
// and none more than kMaxCellWarp, the big-cell tiles when some cell holds
// more than kMaxCell.  Results do not depend on the form.
constexpr uint32_t kFormTile = 0u, kFormBig = 1u, kFormCell = 2u;
constexpr uint32_t kDenseCell = 24u;
constexpr int kMaxCellWarp = 256;        // agents per cell of the warp-per-cell kernels
// dense: the mean occupancy of the non-empty cells from which the
// warp-per-cell form runs (kDenseCell unless a batch's launch tuning sets it)
__host__ __device__ inline uint32_t step_form(uint32_t max_cell, uint32_t n_agents, uint32_t n_nonempty,
                                              uint32_t dense = kDenseCell) {
    if (max_cell > (uint32_t)kMaxCell) return kFormBig;
    if (max_cell > (uint32_t)kMaxCellWarp) return kFormTile;
    return ((uint64_t)n_agents >= (uint64_t)dense * n_nonempty) ? kFormCell : kFormTile;
}
// bytes every agent column is allocated beyond its rows: bulk copies read
// whole 16-byte units around a row range
constexpr size_t kColumnPad = 64;
constexpr int kScanThreads = 256;
// cells per thread in the cell scan: one for grids of up to kScanWideCells
// cells, two above (fewer look-back steps pay off on the larger grids);
// tile-status arrays are sized for one cell per thread
constexpr int kScanItems = 1;
constexpr int kScanTile = kScanThreads * kScanItems;
constexpr int kScanWideCells = 4 << 20;
__host__ __device__ inline int scan_items(int num_cells) { return num_cells > kScanWideCells ? 2 : 1; }
constexpr int kStatsRing = 1024;
constexpr int kBatchRing = 64;           // per-run statistics ring of a batch (steps)
constexpr uint32_t kNoRun = 0xffffffffu; // run index of a batch cell that belongs to no run
constexpr uint8_t kStagedDead = 0xffu;   // meta byte of a staged row that is not admitted
constexpr uint32_t kSpinLimit = 1u << 26;  // bounded waits in the look-back (polls)
constexpr uint64_t kWaitLimitNs = 1000000000ull;  // ... and their time limit (1 s)

// random stream bases (Philox counter word 0), see oracle/philox4x32.h
constexpr uint32_t kStreamActions = 0u;
constexpr uint32_t kStreamPair = 64u;
constexpr uint32_t kStreamBirth = 128u;

// genetics: at most 64 blocks of 64 loci per strand, Poisson(1) counts capped
// at 16, and at most 128 draws of the birth stream per newborn
constexpr int kMaxGenomeBlocks = 64;
constexpr int kMaxBinomial = 64;
constexpr int kBirthDraws = 128;
constexpr int kMaxFixedCrossover = 30;   // 3 + 2*30 + 1 + 64 draws fit kBirthDraws
constexpr int kCrossoverPoisson1 = -100;

// life states of the downloaded table (QHG_LS_ALIVE, QHG_LS_FERTILE)
constexpr uint8_t QHG_LS_ALIVE_DEV = 1u, QHG_LS_FERTILE_DEV = 5u;

// agent meta byte: bit 0 gender, bit 1 fertile (life state 5, else 1)
constexpr uint8_t kMetaGender = 1u;
constexpr uint8_t kMetaFertile = 2u;

// outcome byte of a step: bits 0-2 class (0 dead, 1 stay, 2..7 moved to
// neighbour slot class-2), bit 3 gives birth, bit 4 fertile, bit 5 gender
constexpr uint8_t kOutBirth = 8u;
constexpr uint8_t kOutFertile = 16u;
constexpr uint8_t kOutGender = 32u;
constexpr uint8_t kOutMoved = 64u;    // registered a move (statistics only)
constexpr uint8_t kOutDropped = 128u; // left with its run (batches): not a death

// per-cell class counts: [0] stay, [1..6] movers per neighbour slot, [7] births
constexpr int kCls = 8;

enum ActionType : int32_t {
    kGetOld = 0, kFertility = 1, kRandomPair = 2, kVerhulst = 3, kVerhulstVarK = 4,
    kOldAgeDeath = 5, kRandomMove = 6, kWeightedMove = 7, kATanDeath = 8
};

// ATanDeath (actions/ATanDeath.h, utils/qhg_consts.h): EPS of its scale and
// Q_PI = std::numbers::pi, the double nearest pi
constexpr double kATanEps = 0.001;
constexpr double kQPi = 3.141592653589793;

enum ErrorCode : uint32_t {
    kErrNone = 0, kErrCellTooLarge = 1, kErrTimeout = 2, kErrCapacity = 3, kErrInternal = 4, kErrBadCell = 5
};

// constants of one action, prepared on the host
struct ActionConst {
    int32_t type;
    uint32_t window;        // first draw of the action in the per-agent stream
    int32_t vslot;          // Verhulst: index among the population's Verhulst actions
    float f0, f1, f2;       // Fertility: min age, max age, interbirth
    float age_lo, age_hi;   // OldAgeDeath, ATanDeath: float bounds of the uncertain age window
    double b0, d0, th;      // Verhulst
    double th_b0, th_d0;    // theta - b0, theta - d0
    double K;               // Verhulst constant K
    double oad_M, oad_a, oad_w;  // OldAgeDeath: max age, 1 - U*M, (1+U*M) - (1-U*M)
    double at_M, at_slope, at_scale;  // ATanDeath: max age, slope, (pi/2 - EPS) / atan(slope * range)
    uint64_t pthr;          // RandomMove / WeightedMove: u < pthr  <=>  u/2^32 < p
};

struct StepConst {
    uint64_t seed;
    uint32_t rkey[20];       // Philox round keys of the seed (philox_round_keys)
    int32_t n_act;
    int32_t age_from_birth;  // GetOld or OldAgeDeath runs: a survivor's age is t - birth
    int32_t has_pair;
    int32_t num_cells;
    int32_t log_births;
    int32_t genome_words;    // 2 * blocks, 0 without genetics
    int32_t genome_size;     // loci per strand
    int32_t num_crossover;   // > 0 fixed count, 0 none, kCrossoverPoisson1
    int32_t has_mutation;    // mutation rate > 0
    int32_t n_binomial;      // entries of the mutation-count table
    uint32_t genome_capacity;  // genome slots
    // BinomialDist::getN as integer thresholds: the count is the first i
    // with u <= bino[i] (u the 32-bit draw), n_binomial if none; bino[i] =
    // floor(L_i * 2^32) of the table entry L_i, so u / 2^32 > L_i <=> u > bino[i]
    int64_t bino[kMaxBinomial];
    uint32_t capacity;
    int32_t reads_age;       // some action reads the stored age before GetOld/OldAgeDeath sets it
    int32_t n_verhulst;
    int32_t verhulst_act[kMaxVerhulst];
    int32_t program;         // specialised action program (0: interpreted)
    int32_t has_move;        // RandomMove or WeightedMove present
    int32_t has_wmove;       // WeightedMove present
    uint32_t dense_cell;     // mean occupancy from which a step runs the warp-per-cell form (step_form)
    ActionConst act[kMaxActions];
};

// per-run scalars in device memory
struct RunState {
    int32_t step;            // time of the next step is (float)step
    uint32_t n_agents;
    int64_t next_id;
    uint32_t n_nonempty;
    uint32_t error;          // first error (ErrorCode)
    uint32_t error_info;
    uint32_t scan_tiles_started;
    uint32_t scatter_ctas_done;
    uint32_t action_tiles;    // tiles handed out by k_actions
    uint32_t scatter_tiles;   // tiles handed out by k_scatter
    // written by the cell scan, committed when the scatter finishes
    uint32_t new_n_agents;
    uint32_t new_n_nonempty;
    uint32_t births;
    uint64_t birth_log_n;
    // genome slots: the free list of the current step (slots of agents that
    // died in the previous step, plus unused ones carried over) and the
    // high-water mark of never used slots
    uint32_t nfree;
    uint32_t hwm;
    uint32_t dead_count;     // deaths of this step pushed to the next free list
    int32_t genome_step;     // step whose newborns k_genomes builds
    uint32_t n_staged;       // batches: agents waiting to be placed by k_inject
    uint32_t form;           // kernels of the step (kFormTile, kFormBig, kFormCell)
    uint32_t form_next;      // the same for the table the step writes (set by its commit)
    uint32_t max_cell;       // largest cell of the next table when above kMaxCellWarp (cell scan)
    uint32_t stall_tile;     // tests of the bounded waits: tile + 1 whose scan status is withheld once
    // single runs whose actions set every survivor's age to t - birth
    // (GetOld or OldAgeDeath): once a step has run, the table's age column is
    // not kept up to date; its ages are (float)(step - 1) - birth
    uint32_t age_derived;
    // statistics ring: [step % kStatsRing][live, births, deaths, moves]
    unsigned long long stats[kStatsRing][4];
};

// device pointers of one step: the current table, the next table, the
// grid and the step's scratch arrays
struct StepBuffers {
    // current table: non-empty cells in index order and the first row of each
    // (ne_start has n_nonempty + 1 entries, the last one the agent count)
    // tile_first[t]: index of the first non-empty cell of tile t (ceil(N/kTileAgents)+1 entries)
    const uint32_t *nonempty; const uint32_t *ne_start; const uint32_t *tile_first;
    const int64_t *id; const float *birth; const float *age; const float *lastb; const uint8_t *meta;
    uint32_t *nonempty2; uint32_t *ne_start2; uint32_t *tile_first2;
    int64_t *id2; float *birth2; float *age2; float *lastb2; uint8_t *meta2;
    // rev packs, 3 bits per neighbour slot q, the slot of this cell in the
    // neighbour's own list
    const int32_t *nbr; const uint8_t *nnbr; const uint32_t *rev; const double *K;
    // Verhulst thresholds of each non-empty cell, by its position in the
    // non-empty list: for this step's table (read by k_actions) and for the
    // next table (written by the scan); kept per table so that a failed step
    // leaves the current ones intact for its retry
    const ulonglong2 *vthr; ulonglong2 *vthr2;
    // moves: WeightedMove thresholds (6 per cell) and one word per cell:
    // bits 0-2 neighbour count, bits 8-13 valid neighbour slots, bit 16 all
    // weights equal
    const uint64_t *wthr; const uint32_t *cmove;
    // the move word of each non-empty cell by its position in the non-empty
    // list (current table, next table), copied from cmove by the cell scan;
    // the Verhulst thresholds above are stored by the same positions
    const uint32_t *necm; uint32_t *necm2;
    // occupancy tracking (single runs with QHG_FLAG_TRACK_OCCUPANCY, else
    // null): per cell, the first step whose table holds an agent there, -1 none
    int32_t *occ;
    // MoveStats (single runs, ms_mode >= 0: 0 first, 1 min, 2 last): per cell
    // the definitive hops, distance and time; this step's candidates (hops,
    // distance as the bits of a non-negative double, mover ID key) per
    // destination cell; the distance to each neighbour slot (cells x 6)
    int32_t ms_mode;
    int32_t *ms_hops; double *ms_dist; double *ms_time;
    int32_t *ms_chops; unsigned long long *ms_cdist; unsigned long long *ms_ckey;
    const double *ms_D;
    // outcome word per agent: outcome byte | local cell << 8 | rank in its
    // cell's class << 17
    uint32_t *outc; int32_t *father; uint16_t *brank; uint32_t *clsc;
    uint32_t *sbase; uint32_t *bbase; uint32_t *bidbase; uint32_t *obase;
    uint32_t *tile_flag; uint4 *tile_agg; uint4 *tile_incl;
    int64_t *blog; uint64_t blog_cap;
    // genetics: genome slot per agent (current, next), the genome slab
    // (genome_capacity x genome_words), free lists (current, next), and one
    // record per newborn by global birth rank: {mother slot, father slot,
    // baby slot, mother ID low, mother ID high}
    const int32_t *gslot; int32_t *gslot2;
    uint64_t *genome;
    const uint32_t *freelist; uint32_t *freelist2;
    uint32_t *brec;
};

// One run of a batch: its seed, the batch step at which its step 0 runs,
// its cell range and its action parameters (the batch's action types and
// draw windows, the run's own values).  Runs with active == 0 leave the
// batch at the next step.
struct BatchRun {
    uint64_t seed;
    int32_t step0;
    uint32_t active;
    uint32_t cell0, cell1;
    ActionConst act[kMaxActions];
};

// device pointers of a batch step (in addition to StepBuffers)
struct BatchBuffers {
    const uint32_t *crun;       // run of each cell (kNoRun: free)
    const BatchRun *runs;
    int64_t *rnext;             // next agent ID of each run
    // per run and ring slot (batch step % kBatchRing): live, births, deaths, moves
    uint32_t *rstat;
    int32_t nruns;              // run slots in use (upper bound of run indices)
    // admission: staged agents (any order), their count per cell; placed by
    // k_inject after the scatter
    uint32_t *inj;
    uint32_t *ibase;
    const int64_t *sid; const float *sbirth; const float *sage; const float *slastb;
    const uint8_t *smeta; const uint32_t *scell;
    uint32_t *inj_ctas_done;
    uint32_t *cstat;            // per cell: deaths | registered moves << 16 of the step
};

// grid sizes of the persistent tile kernels (CTAs); results do not depend
// on them (tiles are dealt out statically, draws are keyed by agent ID)
struct LaunchShape {
    int actions_grid;
    int scatter_grid;
    int big_grid;      // CTAs of the big-cell forms (one per SM)
    int scan_items;    // cells per thread of the cell scan (1 or 2; 0: chosen from the grid size)
};

// ------------------------------------------------------------- Philox
struct Draw4 { uint32_t v[4]; };

constexpr uint32_t kPhiloxM0 = 0xD2511F53u, kPhiloxM1 = 0xCD9E8D57u;
constexpr uint32_t kPhiloxW0 = 0x9E3779B9u, kPhiloxW1 = 0xBB67AE85u;

// Philox4x32-10 (Salmon et al., SC'11); each round's two 32x32-bit products
// are taken as one 64-bit product each (high and low words)
__device__ __forceinline__ Draw4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                               uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        const uint64_t p0 = (uint64_t)kPhiloxM0 * c0;
        const uint64_t p1 = (uint64_t)kPhiloxM1 * c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c0 = n0; c1 = (uint32_t)p1; c2 = n2; c3 = (uint32_t)p0;
        k0 += kPhiloxW0;
        k1 += kPhiloxW1;
    }
    Draw4 d;
    d.v[0] = c0; d.v[1] = c1; d.v[2] = c2; d.v[3] = c3;
    return d;
}

// the same with the ten round keys given (rk[2r], rk[2r+1] for round r)
__device__ __forceinline__ Draw4 philox4x32_10_rk(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                                  const uint32_t *rk) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        const uint64_t p0 = (uint64_t)kPhiloxM0 * c0;
        const uint64_t p1 = (uint64_t)kPhiloxM1 * c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ rk[2 * r];
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ rk[2 * r + 1];
        c0 = n0; c1 = (uint32_t)p1; c2 = n2; c3 = (uint32_t)p0;
    }
    Draw4 d;
    d.v[0] = c0; d.v[1] = c1; d.v[2] = c2; d.v[3] = c3;
    return d;
}

// round keys of a seed (host and device)
__host__ __device__ inline void philox_round_keys(uint64_t seed, uint32_t *rk) {
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    for (int r = 0; r < 10; r++) {
        rk[2 * r] = k0;
        rk[2 * r + 1] = k1;
        k0 += kPhiloxW0;
        k1 += kPhiloxW1;
    }
}

// the block `blk` of the stream (seed, step, id)
__device__ __forceinline__ Draw4 draw_block(uint64_t seed, uint32_t step, int64_t id, uint32_t blk) {
    uint64_t u = (uint64_t)id;
    return philox4x32_10(blk, step, (uint32_t)u, (uint32_t)(u >> 32), (uint32_t)seed, (uint32_t)(seed >> 32));
}

// the block `blk` of an agent's stream: from the run's precomputed round keys
// (a single run: kernel-parameter constants) or from the run's seed (batches)
template <bool BATCH>
__device__ __forceinline__ Draw4 run_block(const StepConst &P, uint64_t seed, uint32_t step, int64_t id,
                                           uint32_t blk) {
    if (BATCH) return draw_block(seed, step, id, blk);
    const uint64_t u = (uint64_t)id;
    return philox4x32_10_rk(blk, step, (uint32_t)u, (uint32_t)(u >> 32), P.rkey);
}

}  // namespace qhg
