/*
 * qhg_gpu.h - C ABI of the GB300 implementation of QHG4's per-step agent
 * hot path (libqhg_gpu.so).
 *
 * One handle (qhg_run) holds one simulation: the cell grid and the agents
 * live in device memory (HBM) between calls.  A step is the reference's
 * PopLooper::doStep (core/PopLooper.cpp:166-200) for one population:
 * initializeStep (rates, pairing), doActions over all priority levels,
 * finalizeStep (births, deaths, moves, per-cell counts).
 *
 * The entry points replace, in the reference:
 *   qhg_gpu_create         SPopulation<T>::SPopulation + the action objects and
 *                          Prioritizer set-up (core/SPopulation.cpp:44-84,
 *                          core/SPopulation.cpp:247-261 setPrioList,
 *                          populations/tut_SexualPop.cpp:24-43)
 *   qhg_gpu_upload_grid    SCellGrid neighbour table (core/SCellGrid.h:45-57,
 *                          core/SCell.h:4-12) and the K / weight arrays
 *                          (actions/VerhulstVarK.cpp:29, actions/SingleEvaluator.cpp:174-241)
 *   qhg_gpu_upload_agents  SPopulation<T>::addAgent / setAgentBasic
 *                          (core/SPopulation.cpp:1149, 1254) for a whole table
 *   qhg_gpu_step           PopLooper::doStep (core/PopLooper.cpp:166-200):
 *                          SPopulation<T>::initializeStep (core/SPopulation.cpp:394),
 *                          doActions (:554), finalizeStep (:439) with
 *                          recycleDeadSpaceNew (:596), performMoves (:1058),
 *                          updateNumAgentsPerCell (:509)
 *   qhg_gpu_download       the agent table as SPopulation<T>::writeAgentDataQDFSafe
 *                          (core/SPopulation.cpp:1465) collects it
 *   qhg_gpu_counts         SPopulation<T>::getNumAgentsArray (core/SPopulation.h:142)
 *   qhg_gpu_destroy        SPopulation<T>::~SPopulation (core/SPopulation.cpp:94)
 *
 * Rules: every call returns an int status (QHG_OK = 0, negative = error;
 * qhg_gpu_last_error() describes the last error of the calling thread).
 * Buffers passed in are host memory owned by the caller and are not kept.
 * A handle is used by one host thread at a time.  Nothing throws across the
 * ABI.  Random draws are Philox4x32-10 keyed by (seed, step, agent ID,
 * action), so results do not depend on launch shapes or memory layout.
 */
#ifndef QHG_GPU_H
#define QHG_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define QHG_OK                  0
#define QHG_ERR_ARG            -1   /* invalid argument */
#define QHG_ERR_CUDA           -2   /* CUDA runtime error */
#define QHG_ERR_NOMEM          -3   /* device or host allocation failed */
#define QHG_ERR_STATE          -4   /* call out of order (e.g. step before upload) */
#define QHG_ERR_CELL_TOO_LARGE -5   /* a cell holds more agents than QHG_MAX_CELL_AGENTS */
#define QHG_ERR_TIMEOUT        -6   /* a device-side wait gave up (bounded spin) */
#define QHG_ERR_CAPACITY       -7   /* agent or genome capacity exhausted */
#define QHG_ERR_DEVICE         -8   /* a kernel reported an inconsistency */

/* action type codes (reference class names in parentheses) */
#define QHG_ACT_GETOLD        0  /* GetOld        actions/GetOld.cpp:37-48 */
#define QHG_ACT_FERTILITY     1  /* Fertility     actions/Fertility.cpp:49-73 */
#define QHG_ACT_RANDOMPAIR    2  /* RandomPair    actions/RandomPair.cpp:107-270 */
#define QHG_ACT_VERHULST      3  /* Verhulst      actions/Verhulst.cpp:70-121 */
#define QHG_ACT_VERHULSTVARK  4  /* VerhulstVarK  actions/VerhulstVarK.cpp:69-111 */
#define QHG_ACT_OLDAGEDEATH   5  /* OldAgeDeath   actions/OldAgeDeath.cpp:48-67 */
#define QHG_ACT_RANDOMMOVE    6  /* RandomMove    actions/RandomMove.cpp:65-100 */
#define QHG_ACT_WEIGHTEDMOVE  7  /* WeightedMove  actions/WeightedMove.cpp:45-106 */
#define QHG_ACT_ATANDEATH     8  /* ATanDeath     actions/ATanDeath.cpp:41, 57-77 */

#define QHG_MAX_ACTIONS       16
#define QHG_MAX_CELL_AGENTS   4608   /* agents one cell may hold */
#define QHG_CROSSOVER_POISSON1 (-100) /* Poisson(1) breakpoints per parent */

/* life states stored in the agent table (core/SPopulation.h:69-73) */
#define QHG_LS_ALIVE          1
#define QHG_LS_FERTILE        5

/* flags of qhg_run_desc */
#define QHG_FLAG_LOG_BIRTHS   1u   /* keep a (baby, mother, father) ID log */
#define QHG_FLAG_TRACK_OCCUPANCY 2u /* record when each cell is first occupied (qhg_gpu_occupancy) */

typedef struct qhg_run qhg_run;

/*
 * Description of one population.  Actions are given in execution order:
 * ascending priority, ties in alphabetical order of the reference class
 * name (the order SPopulation::setPrioList produces).  Parameter slots:
 *   FERTILITY     {min_age, max_age, interbirth}
 *   VERHULST      {b0, d0, theta, K}
 *   VERHULSTVARK  {b0, d0, theta}            (K per cell from the grid)
 *   OLDAGEDEATH   {max_age, uncertainty}
 *   ATANDEATH     {max_age, range, slope}
 *   RANDOMMOVE    {prob}
 *   WEIGHTEDMOVE  {prob}                     (weights: the grid's K, cumulated)
 */
typedef struct {
    uint64_t seed;
    int32_t  n_actions;
    int32_t  action_type[QHG_MAX_ACTIONS];
    double   action_param[QHG_MAX_ACTIONS][4];
    int32_t  genome_size;      /* loci per strand, 0 = no genetics */
    int32_t  num_crossover;    /* > 0 fixed count, 0 none, QHG_CROSSOVER_POISSON1 */
    double   mutation_rate;    /* per locus */
    int64_t  agent_capacity;   /* agent slots to allocate (0: 4 x initial + 65536) */
    uint32_t flags;            /* QHG_FLAG_* */
    int32_t  device;           /* CUDA device ordinal */
} qhg_run_desc;

/* agent table, structure of arrays; genome is n x (2 * ceil(genome_size/64))
 * words, strand 0 then strand 1 (actions/Genetics.h m_aGenome layout) */
typedef struct {
    int64_t  *id;
    int32_t  *cell;
    float    *birth;
    float    *age;
    float    *last_birth;
    uint8_t  *gender;
    uint8_t  *state;
    uint64_t *genome;
} qhg_agents_soa;

/* per-step statistics */
typedef struct {
    uint64_t live;     /* agents alive after the step */
    uint64_t births;
    uint64_t deaths;
    uint64_t moves;    /* registered moves */
} qhg_step_stats;

const char *qhg_gpu_last_error(void);
const char *qhg_gpu_version(void);

int qhg_gpu_create(const qhg_run_desc *desc, qhg_run **out);
int qhg_gpu_upload_grid(qhg_run *run, const int32_t *nbr6, const uint8_t *nnbr, const double *K,
                        int32_t num_cells);
/* Environment updates between steps, for populations whose K and move
 * weights come from environment evaluators (populations/FlatExpPop.cpp:43-56):
 * qhg_gpu_set_capacity takes a new K per cell (C entries), what NPPCapacity
 * writes into the capacity array (actions/NPPCapacity.cpp) and VerhulstVarK
 * reads at each step's initialize (actions/LinearBirth.cpp:90-112,
 * actions/LinearDeath.cpp:92-122); unless weights were given, WeightedMove's
 * weights follow K as after qhg_gpu_upload_grid.  qhg_gpu_set_move_weights
 * takes WeightedMove's cumulative weights (C x 7: W[c][0] the cell's own
 * weight, W[c][i+1] = W[c][i] + neighbour i's), what MultiEvaluator /
 * SingleEvaluator leave in the weight array (actions/MultiEvaluator.cpp:221-255,
 * actions/SingleEvaluator.cpp:174-241) and WeightedMove reads
 * (actions/WeightedMove.cpp:57-80); from then on they no longer follow K.
 * A row whose W[c][0] differs from W[c][n] (n neighbours) must have finite
 * entries and W[c][n] > 0 (QHG_ERR_ARG otherwise).  Both wait for the run's
 * stream, report a device-side error of an earlier step like qhg_gpu_sync
 * (and then change nothing), and take effect from the next step on. */
int qhg_gpu_set_capacity(qhg_run *run, const double *K);
int qhg_gpu_set_move_weights(qhg_run *run, const double *cumw7);
/* The ice flags of the grid's Geography (Geography::m_abIce, C entries,
 * nonzero = ice; NULL = no ice), from the next step on: WeightedMove
 * registers no move into an ice cell (actions/WeightedMove.cpp:91; its draws
 * are taken all the same), and weights that follow K give ice cells weight
 * 0, as the SingleEvaluator does (actions/SingleEvaluator.cpp:183-202).
 * RandomMove ignores ice, as in the reference.  qhg_gpu_upload_grid clears
 * the flags.  Waits for the run's stream like qhg_gpu_set_capacity. */
int qhg_gpu_set_ice(qhg_run *run, const uint8_t *ice);
/* agents in any order; dead rows (state 0) are dropped */
int qhg_gpu_upload_agents(qhg_run *run, const qhg_agents_soa *agents, int64_t n, int32_t first_step);
/* runs nsteps steps asynchronously on the run's stream */
int qhg_gpu_step(qhg_run *run, int32_t nsteps);
/* waits for the run's stream and reports device-side errors */
int qhg_gpu_sync(qhg_run *run);
int qhg_gpu_num_agents(qhg_run *run, int64_t *n);
int qhg_gpu_current_step(qhg_run *run, int32_t *step);
/* agents ordered by cell (device order); cap = room in the caller's arrays */
int qhg_gpu_download(qhg_run *run, qhg_agents_soa *out, int64_t cap, int64_t *n);
int qhg_gpu_counts(qhg_run *run, uint32_t *cell_counts);
/* statistics of the last `nsteps` steps (nsteps <= 1024) */
int qhg_gpu_stats(qhg_run *run, int32_t nsteps, qhg_step_stats *out);
/* Queues on the run's stream a copy of the statistics of the step launched
 * last into *out and returns without waiting (the per-step counts that
 * PopLooper reads from the population after each step,
 * core/PopLooper.cpp:166-200; *out should be page-locked host memory, see
 * qhg_host_buffer_alloc).  The values are there once qhg_gpu_sync (or any
 * call that waits for the run) has returned; a step that failed leaves
 * undefined values and its error is reported by that call. */
int qhg_gpu_stats_async(qhg_run *run, qhg_step_stats *out);
/* Occupation history of the cells (QHG_FLAG_TRACK_OCCUPANCY): per cell the
 * first step whose table holds an agent there (the uploaded table counts as
 * its step), -1 if none yet; C entries.  Replaces OccTracker::updateCounts
 * with OccHistory::addEntry (core/OccTracker.cpp, core/OccHistory.cpp) for
 * one population: occupation masks that change to non-zero are recorded,
 * masks of zero are ignored. */
int qhg_gpu_occupancy(qhg_run *run, int32_t *first_step);
/* Restores the occupation history (C entries as qhg_gpu_occupancy gives
 * them) after a checkpoint's table was uploaded. */
int qhg_gpu_set_occupancy(qhg_run *run, const int32_t *first_step);
/* MoveStats (actions/MoveStats.cpp, actions/MoveStats.h): per cell the hops,
 * the distance travelled and the time of arrival of the agents that reached
 * it, with the reference's modes MODE_STAT_FIRST / MIN / LAST:
 *   QHG_MOVESTATS_FIRST  the first arrival (lowest mover ID of the first
 *                        step that reaches the cell)
 *   QHG_MOVESTATS_MIN    fewest hops, shortest distance, time of the first
 *                        arrival
 *   QHG_MOVESTATS_LAST   the latest arrival (highest mover ID of the last
 *                        step with arrivals)
 * A move from f to t offers hops[f] + 1 and dist[f] + d(f, t), as
 * MoveStats::finalize does on one thread (its per-thread merge makes more
 * threads order-dependent), with moves in agent-ID order instead of slot
 * order; every registered move counts, also one whose agent a later action
 * of the step killed.  Distances: spherdistDeg over the cells' lon/lat in
 * degrees on a sphere of `radius`, or cartdist over x = lon, y = lat when
 * `cartesian` (utils/geomutils.cpp:311-386).  Enabling (re)starts the
 * statistics from the current table (MoveStats::initializeOccupied: its
 * cells 0, the others -1) and so does each later qhg_gpu_upload_agents.
 * qhg_gpu_move_stats copies C entries each.  Single runs only. */
#define QHG_MOVESTATS_FIRST   0
#define QHG_MOVESTATS_MIN     1
#define QHG_MOVESTATS_LAST    2
int qhg_gpu_move_stats_enable(qhg_run *run, int32_t mode, const double *lon, const double *lat, double radius,
                              int32_t cartesian);
int qhg_gpu_move_stats(qhg_run *run, int32_t *hops, double *dist, double *time);
/* Restores the statistics (as qhg_gpu_move_stats gives them) after a
 * checkpoint's table was uploaded and MoveStats enabled: the reference's
 * MoveStats::readAdditionalDataQDF (actions/MoveStats.cpp) on --resume. */
int qhg_gpu_set_move_stats(qhg_run *run, const int32_t *hops, const double *dist, const double *time);
/* birth log (QHG_FLAG_LOG_BIRTHS): rows (baby, mother, father) */
int qhg_gpu_birth_log(qhg_run *run, int64_t *baby, int64_t *mother, int64_t *father, int64_t cap,
                      int64_t *n);
/* The next agent ID the run gives out (IDGen::getID, core/IDGen.h:28).
 * Checkpoint/resume (the reference's dumpSpeciesDataQDF and --resume,
 * core/SPopulation.cpp:2138, app/SimParams.cpp:357): the state of a run is
 * its agent table, its step and this counter; qhg_gpu_upload_agents with
 * first_step = the saved step followed by qhg_gpu_set_next_id restores it,
 * and the resumed run continues exactly as the uninterrupted one.  The ID
 * must exceed every live agent's ID; set it after the upload, before a step. */
int qhg_gpu_next_id(qhg_run *run, int64_t *next_id);
int qhg_gpu_set_next_id(qhg_run *run, int64_t next_id);
/* For tests of failure detection: the next step's cell scan withholds the
 * status of scan tile `tile` (cells tile*512 ..), so that the look-back of
 * the tile after it waits until its limit (about one second), gives up and
 * the step fails with QHG_ERR_TIMEOUT -- reported by the next qhg_gpu_sync;
 * the run keeps its last step and can be stepped again.  Nothing faults or
 * hangs: every device-side wait of the library is bounded this way.  The
 * grid must have more than 512 cells; tile < (cells + 511) / 512 - 1. */
int qhg_gpu_test_stall_scan(qhg_run *run, int32_t tile);
/* the run's CUDA stream (cudaStream_t) */
int qhg_gpu_stream(qhg_run *run, void **stream);
int qhg_gpu_destroy(qhg_run *run);

/*
 * Runs nsteps steps like qhg_gpu_step, but launches each kernel on its own
 * (no CUDA graph) between CUDA events on the run's stream and waits for
 * each step.  kernel_ms (nsteps x 4) receives the device time of each
 * kernel of each step: actions, cell scan, scatter, genomes (0 without
 * genetics).  For measurement only.
 */
int qhg_gpu_step_profiled(qhg_run *run, int32_t nsteps, float *kernel_ms);

/* runs nsteps steps like qhg_gpu_step between two CUDA events recorded on
 * the run's stream, waits, and returns the device time in *elapsed_ms */
int qhg_gpu_step_timed(qhg_run *run, int32_t nsteps, float *elapsed_ms);

/* ------------------------------------------------------------------------
 * Batches: many independent runs of one action list in one device table,
 * stepped together (one launch of each step kernel over all runs, captured
 * as a CUDA graph).  Runs differ in seed, grid, population and action
 * parameters; every run's results are the same as those of the run alone
 * through qhg_gpu_* with the same inputs.  Runs can join (qhg_batch_add_run)
 * and leave (qhg_batch_remove_run) between steps: this is what served
 * execution builds on.  The reference has no batched form: a QHG4 process
 * runs one simulation; these calls replace running qhg_gpu_* (or the
 * reference) once per simulation.
 * ------------------------------------------------------------------------ */
typedef struct qhg_batch qhg_batch;

typedef struct {
    int32_t  n_actions;                         /* action types in execution order (as qhg_run_desc) */
    int32_t  action_type[QHG_MAX_ACTIONS];
    int64_t  agent_capacity;                    /* rows of the shared agent table */
    int64_t  cell_capacity;                     /* cells of all runs in the batch at once */
    int64_t  stage_capacity;                    /* agents admitted between two steps */
    int32_t  max_runs;                          /* runs in the batch at once */
    int32_t  device;
} qhg_batch_desc;

typedef struct {
    uint64_t seed;
    double   action_param[QHG_MAX_ACTIONS][4];  /* this run's parameters (slots as qhg_run_desc) */
} qhg_batch_run_desc;

typedef struct {
    int32_t active;       /* 0 once removed */
    int32_t cell0;        /* first cell of the run in the batch's cell space */
    int32_t num_cells;
    int32_t steps_done;   /* steps the run has executed */
} qhg_batch_run_status;

const char *qhg_batch_last_error(void);
int qhg_batch_create(const qhg_batch_desc *desc, qhg_batch **out);
/* admits a run (grid as qhg_gpu_upload_grid, agents as qhg_gpu_upload_agents
 * with first step 0); its agents enter at the next qhg_batch_step, after
 * which it has done 0 steps.  *run receives its index. */
int qhg_batch_add_run(qhg_batch *batch, const qhg_batch_run_desc *run_desc, const int32_t *nbr6,
                      const uint8_t *nnbr, const double *K, int32_t num_cells, const qhg_agents_soa *agents,
                      int64_t n, int32_t *run);
/* the run's agents leave at the next step; read its results before */
int qhg_batch_remove_run(qhg_batch *batch, int32_t run);
int qhg_batch_step(qhg_batch *batch, int32_t nsteps);
int qhg_batch_step_timed(qhg_batch *batch, int32_t nsteps, float *elapsed_ms);
int qhg_batch_sync(qhg_batch *batch);
int qhg_batch_num_agents(qhg_batch *batch, int64_t *n);
int qhg_batch_run_info(qhg_batch *batch, int32_t run, qhg_batch_run_status *info);
/* statistics of the run's last nsteps steps (nsteps <= 64) */
int qhg_batch_stats(qhg_batch *batch, int32_t run, int32_t nsteps, qhg_step_stats *out);
/* agents of all runs after each of the batch's last nsteps steps (<= 1024) */
int qhg_batch_live_history(qhg_batch *batch, int32_t nsteps, uint64_t *live);
/* the run's agents ordered by cell, cells relative to the run's grid */
int qhg_batch_download(qhg_batch *batch, int32_t run, qhg_agents_soa *out, int64_t cap, int64_t *n);
int qhg_batch_counts(qhg_batch *batch, int32_t run, uint32_t *cell_counts);
/* Starts copying the run's current table into the caller's buffers on a
 * copy stream and returns without waiting for the copy (the buffers should
 * be page-locked for that); *n receives the rows, *run_step the run's steps
 * done.  The next batch step overlaps the copy; the one after waits for it.
 * Unlike qhg_batch_download, `cell` receives cells of the batch's cell space
 * (uint32, subtract the run's cell0) and `state` the raw meta byte (bit 0
 * gender, bit 1 FERTILE); `gender` is not written.  Call
 * qhg_batch_snapshot_wait before reading the buffers. */
int qhg_batch_snapshot_async(qhg_batch *batch, int32_t run, qhg_agents_soa *out, int64_t cap, int64_t *n,
                             int32_t *run_step);
int qhg_batch_snapshot_wait(qhg_batch *batch);
/* page-locked host memory for qhg_batch_snapshot_async (errors through
 * qhg_batch_last_error) */
int qhg_host_buffer_alloc(int64_t bytes, void **out);
int qhg_host_buffer_free(void *p);
/* launch shape of the persistent kernels (CTAs per SM); results do not
 * depend on it */
int qhg_batch_set_shape(qhg_batch *batch, int32_t actions_ctas_per_sm, int32_t scatter_ctas_per_sm);
int qhg_batch_get_shape(qhg_batch *batch, int32_t *actions_ctas_per_sm, int32_t *scatter_ctas_per_sm,
                        int32_t *max_actions, int32_t *max_scatter);
/* The batch's launch tuning (what its autotuner searches; results do not
 * depend on it): CTAs per SM of the action kernel and of the scatter, cells
 * per thread of the cell scan (1 or 2; 0: chosen from the grid size), and
 * the mean occupancy of the non-empty cells from which a step runs the
 * warp-per-cell form instead of cell-aligned tiles (0: the default, 24).
 * Waits for the batch; the form threshold applies from the next step's
 * commit on. */
typedef struct {
    int32_t actions_ctas_per_sm;
    int32_t scatter_ctas_per_sm;
    int32_t scan_cells_per_thread;
    int32_t dense_cell;
} qhg_batch_launch;
int qhg_batch_set_launch(qhg_batch *batch, const qhg_batch_launch *launch);
int qhg_batch_get_launch(qhg_batch *batch, qhg_batch_launch *launch);
/* agents and non-empty cells of the batch's table (waits for the batch) */
int qhg_batch_table_info(qhg_batch *batch, int64_t *n_agents, int64_t *n_nonempty_cells);
/* Environment updates of one run between steps, with the effect the
 * single-run calls have on a run alone (qhg_gpu_set_capacity,
 * qhg_gpu_set_move_weights, qhg_gpu_set_ice: NPPCapacity's K,
 * MultiEvaluator's move weights, the Geography's ice, handed over after an
 * environment event, populations/FlatExpPop.cpp:43-56,
 * actions/WeightedMove.cpp:91); arrays cover the run's own grid.  Wait for
 * the batch; QHG_ERR_STATE for a run that has left. */
int qhg_batch_set_capacity(qhg_batch *batch, int32_t run, const double *K);
int qhg_batch_set_move_weights(qhg_batch *batch, int32_t run, const double *cumw7);
int qhg_batch_set_ice(qhg_batch *batch, int32_t run, const uint8_t *ice);
/* Occupation history of every run (as qhg_gpu_occupancy for a run alone,
 * OccTracker::updateCounts, core/OccTracker.cpp): per cell of the run's
 * grid the first of the run's steps whose table holds an agent there (0:
 * the agents it was admitted with), -1 never.  Enable before the first run
 * is added (QHG_ERR_STATE after); it adds one kernel per step over the
 * non-empty cells.  qhg_batch_occupancy waits for the batch. */
int qhg_batch_enable_occupancy(qhg_batch *batch);
int qhg_batch_occupancy(qhg_batch *batch, int32_t run, int32_t *first_step);
/* MoveStats of every run (as qhg_gpu_move_stats_enable / qhg_gpu_move_stats
 * for a run alone, actions/MoveStats.cpp): one mode, radius and distance
 * kind for the batch, enabled before the first run is added
 * (QHG_ERR_STATE after).  A run's state starts at its admission (the cells
 * its agents start in are the origins: hops, distance and time 0); its cell
 * coordinates (lon/lat in degrees, or x/y with cartesian) are given by
 * qhg_batch_move_stats_coords before the steps whose moves should add
 * distances (until then they add 0).  Times are the run's own steps.  Both
 * calls wait for the batch. */
int qhg_batch_move_stats_enable(qhg_batch *batch, int32_t mode, double radius, int32_t cartesian);
int qhg_batch_move_stats_coords(qhg_batch *batch, int32_t run, const double *lon, const double *lat);
int qhg_batch_move_stats(qhg_batch *batch, int32_t run, int32_t *hops, double *dist, double *time);
int qhg_batch_stream(qhg_batch *batch, void **stream);
int qhg_batch_destroy(qhg_batch *batch);

/*
 * Per-cell census of a caller-owned agent table, for callers that cannot
 * allocate device memory (a host runtime with its own fixed device pool, a
 * real-time loop that must not hit cudaMalloc/cudaFree, a device whose heap
 * is exhausted).  This entry point has no counterpart in the reference.
 *
 * d_agent_cell: device array of n_agents cell indices (any order);
 * d_counts (num_cells) receives the live agents per cell and d_first_row
 * (num_cells + 1) the exclusive prefix of the counts, i.e. the first row of
 * each cell in a table sorted by cell, with the agent count last.  Runs on
 * `stream` (a cudaStream_t, NULL for the default stream) on the current
 * device and is synchronous: it reads its error word back to the host and
 * waits for the stream before it returns, so it cannot be called on a
 * stream that is being captured.
 *
 * It allocates nothing: its scratch (the look-back status words) is a
 * file-scope __device__ array sized for QHG_CENSUS_MAX_CELLS cells, held by
 * every GPU that loads the library until the process exits.  Larger grids
 * are rejected with QHG_ERR_ARG.  Every call looks up the array's device
 * address on the current device (cudaGetSymbolAddress, no allocation).  All
 * calls on a device share the array and each leaves its contents behind:
 * calls that overlap on the GPU race and must be serialised by the caller.
 */
#define QHG_CENSUS_MAX_CELLS  4194304
int qhg_gpu_cell_census_noalloc(const int32_t *d_agent_cell, int64_t n_agents, int32_t num_cells,
                                uint32_t *d_counts, uint32_t *d_first_row, void *stream);
/* the last error of qhg_gpu_cell_census_noalloc on the calling thread */
const char *qhg_gpu_census_last_error(void);

#ifdef __cplusplus
}
#endif

#endif
