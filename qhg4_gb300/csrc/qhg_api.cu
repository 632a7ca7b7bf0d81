// Host side of the C ABI declared in include/qhg_gpu.h.
//
// Compiled with -ffp-contract=off: the per-action constants below (the
// OldAgeDeath window, the move-probability thresholds, the WeightedMove
// weight thresholds) must round exactly like the reference's expressions.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "qhg_device.cuh"
#include "qhg_host.h"
#include "../../include/qhg_gpu.h"

extern "C" int qhg_launch_step(const qhg::StepConst *P, qhg::RunState *rs, const qhg::StepBuffers *B,
                               const qhg::BatchBuffers *BB, const qhg::LaunchShape *L, cudaStream_t stream);
extern "C" void qhg_tile_ctas_per_sm(int *actions, int *scatter);
extern "C" int qhg_match_program(const int32_t *types, int n);
extern "C" int qhg_launch_occupancy(const qhg::RunState *rs, const uint32_t *nonempty, int32_t *occ, int grid,
                                    cudaStream_t stream);
extern "C" uint32_t qhg_program_window(int p, int a);
extern "C" int qhg_launch_download_cols(const uint32_t *nonempty, const uint32_t *ne_start, uint32_t nne, uint32_t n,
                                        const uint8_t *meta, const float *birth, float t_prev, int derived,
                                        int32_t *cell_out, uint8_t *gender_out, uint8_t *state_out, float *age,
                                        cudaStream_t stream);
extern "C" int qhg_launch_gather_genomes(const int32_t *gslot, const uint64_t *genome, uint32_t n, int words,
                                         uint32_t slots, uint64_t *out, cudaStream_t stream);
extern "C" int qhg_launch_upload(const qhg::StepConst *P, qhg::RunState *rs, const qhg::StepBuffers *B,
                                 const int32_t *cell, const uint8_t *gender, const uint8_t *state, const int64_t *sid,
                                 const float *sbirth, const float *sage, const float *slastb, int64_t n,
                                 int32_t *gslot_out, cudaStream_t stream);
extern "C" int qhg_launch_step_timed(const qhg::StepConst *P, qhg::RunState *rs, const qhg::StepBuffers *B,
                                     const qhg::BatchBuffers *BB, const qhg::LaunchShape *L, cudaStream_t stream,
                                     cudaEvent_t *ev);

using namespace qhg;

static thread_local std::string g_last_error;

static int fail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

#define CUDA_TRY(expr)                                                                  \
    do {                                                                                \
        cudaError_t e_ = (expr);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            return fail(e_ == cudaErrorMemoryAllocation ? QHG_ERR_NOMEM : QHG_ERR_CUDA, \
                        std::string(#expr) + ": " + cudaGetErrorString(e_));           \
        }                                                                               \
    } while (0)

struct qhg_run {
    qhg_run_desc desc;
    cudaStream_t stream = nullptr;
    StepConst P;
    // grid
    int C = 0;
    int32_t *d_nbr = nullptr;
    uint8_t *d_nnbr = nullptr;
    uint32_t *d_rev = nullptr;
    double *d_K = nullptr;
    ulonglong2 *d_vthr[2] = {nullptr, nullptr};   // per-cell Verhulst thresholds, per table
    std::vector<double> h_K;
    uint64_t *d_wthr = nullptr;
    uint32_t *d_cmove = nullptr;
    int32_t *d_occ = nullptr;       // first step of each cell's occupation (QHG_FLAG_TRACK_OCCUPANCY)
    // MoveStats (qhg_gpu_move_stats_enable): mode (-1 off), state, candidates,
    // distances per cell and neighbour slot
    int32_t ms_mode = -1;
    int32_t *d_ms_hops = nullptr, *d_ms_chops = nullptr;
    double *d_ms_dist = nullptr, *d_ms_time = nullptr, *d_ms_D = nullptr;
    unsigned long long *d_ms_cdist = nullptr, *d_ms_ckey = nullptr;
    std::vector<int32_t> h_nbr;
    std::vector<uint8_t> h_nnbr;
    bool w_given = false;        // move weights given (qhg_gpu_set_move_weights), not from K
    std::vector<uint8_t> h_ice;  // the Geography's ice flags per cell (qhg_gpu_set_ice), empty: none
    int64_t launched = 0;        // steps launched since the run state was last read back
    // agents (ping-pong)
    uint32_t cap = 0;
    int64_t *d_id[2] = {nullptr, nullptr};
    float *d_birth[2] = {nullptr, nullptr};
    float *d_age[2] = {nullptr, nullptr};
    float *d_lastb[2] = {nullptr, nullptr};
    uint8_t *d_meta[2] = {nullptr, nullptr};
    uint32_t *d_ne[2] = {nullptr, nullptr};    // non-empty cells in index order
    uint32_t *d_necm[2] = {nullptr, nullptr};  // their move words, by position in that list
    uint32_t *d_nes[2] = {nullptr, nullptr};   // their first rows (+ agent count)
    uint32_t *d_tf[2] = {nullptr, nullptr};    // first non-empty cell of each tile
    // scratch
    uint32_t *d_outc = nullptr;
    int32_t *d_father = nullptr;
    uint16_t *d_brank = nullptr;
    uint32_t *d_clsc = nullptr, *d_sbase = nullptr, *d_bbase = nullptr, *d_bidb = nullptr, *d_obase = nullptr;
    uint32_t *d_tflag = nullptr;
    uint4 *d_tagg = nullptr, *d_tincl = nullptr;
    int64_t *d_blog = nullptr;
    uint64_t blog_cap = 0;
    // genetics: genome slab indexed by slot, each agent's slot (ping-pong with
    // the table), the free slots (ping-pong) and one record per birth
    uint32_t gcap = 0;
    int32_t *d_gslot[2] = {nullptr, nullptr};
    uint32_t *d_free[2] = {nullptr, nullptr};
    uint64_t *d_genome = nullptr;
    uint32_t *d_brec = nullptr;
    RunState *d_rs = nullptr;
    RunState *h_rs = nullptr;   // pinned
    // step state
    int cur = 0;                 // table holding the current step
    int32_t upload_step = 0;
    int64_t upload_max_id = -1;
    bool grid_ok = false, agents_ok = false;
    LaunchShape shape = {1, 1, 1, 0};
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    std::vector<int64_t> stage;  // host staging for uploads
};

static void free_agents(qhg_run *r) {
    for (int p = 0; p < 2; p++) {
        cudaFree(r->d_id[p]); cudaFree(r->d_birth[p]); cudaFree(r->d_age[p]); cudaFree(r->d_lastb[p]);
        cudaFree(r->d_meta[p]); cudaFree(r->d_ne[p]); cudaFree(r->d_nes[p]); cudaFree(r->d_tf[p]);
        cudaFree(r->d_necm[p]);
        r->d_tf[p] = nullptr; r->d_necm[p] = nullptr;
        r->d_id[p] = nullptr; r->d_birth[p] = r->d_age[p] = r->d_lastb[p] = nullptr;
        r->d_meta[p] = nullptr; r->d_ne[p] = r->d_nes[p] = nullptr;
    }
    cudaFree(r->d_outc); cudaFree(r->d_father); cudaFree(r->d_brank); cudaFree(r->d_blog);
    r->d_outc = nullptr; r->d_father = nullptr; r->d_brank = nullptr; r->d_blog = nullptr;
    for (int p = 0; p < 2; p++) {
        cudaFree(r->d_gslot[p]); cudaFree(r->d_free[p]);
        r->d_gslot[p] = nullptr; r->d_free[p] = nullptr;
    }
    cudaFree(r->d_genome); cudaFree(r->d_brec);
    r->d_genome = nullptr; r->d_brec = nullptr;
    r->gcap = 0;
    r->cap = 0;
}

static void drop_graphs(qhg_run *r) {
    for (int p = 0; p < 2; p++) {
        if (r->graph[p]) cudaGraphExecDestroy(r->graph[p]);
        r->graph[p] = nullptr;
    }
}

// u < thr  <=>  u / 2^32 < x   (exact: u / 2^32 is exact in double)
static uint64_t host_prob_threshold(double x) {
    if (!(x > 0.0)) return 0ull;
    double y = x * 4294967296.0;
    if (y >= 4294967296.0) return 4294967296ull;
    return (uint64_t)std::ceil(y);
}

// largest float f with (double)f <= x
static float float_floor_of(double x) {
    float f = (float)x;
    if ((double)f > x) f = std::nextafter(f, -INFINITY);
    return f;
}

// ATanDeath's death probability (actions/ATanDeath.cpp:62):
// 0.5 + scale * atan(slope * (age - M)) / Q_PI, age promoted from float
static double atan_death_prob(const ActionConst &A, float fa) {
    return 0.5 + A.at_scale * std::atan(A.at_slope * ((double)fa - A.at_M)) / kQPi;
}

// float <-> a key that orders floats like integers (finite and infinite)
static int64_t float_key(float f) {
    int32_t b;
    std::memcpy(&b, &f, 4);
    return b >= 0 ? (int64_t)b : -(int64_t)(b & 0x7fffffff);
}
static float key_float(int64_t k) {
    const int32_t b = k >= 0 ? (int32_t)k : (int32_t)((uint32_t)(-k) | 0x80000000u);
    float f;
    std::memcpy(&f, &b, 4);
    return f;
}

// Ages at which ATanDeath's decision does not depend on the draw.  The
// draw is u / 2^32 with u < 2^32: an agent survives every draw where the
// probability is <= 0 and dies on every draw where it exceeds 1 - 2^-32.
// The probability rises with age when scale * slope > 0; bisection over the
// floats finds age_lo, the oldest age with p <= -delta, and age_hi, the
// oldest age with p < 1 + delta.  The margin delta = 2^-30 is many orders
// above the few ulps by which the device's atan may differ from the host's,
// so ages <= age_lo survive and ages > age_hi die whatever the atan; the
// device evaluates the probability in between.  Without a rising curve, or
// where a bound does not exist, the bound is NaN and the device evaluates
// every age.
static void atan_death_window(ActionConst &A) {
    const float nanf = std::numeric_limits<float>::quiet_NaN();
    A.age_lo = nanf;
    A.age_hi = nanf;
    if (!(std::isfinite(A.at_scale) && std::isfinite(A.at_slope) && std::isfinite(A.at_M) &&
          A.at_scale * A.at_slope > 0))
        return;
    const double delta = 1.0 / 1073741824.0;
    const int64_t kmin = float_key(-INFINITY), kmax = float_key(INFINITY);
    // largest key in [kmin, kmax] whose probability satisfies below(p), given
    // that below holds at kmin and not at kmax
    auto last_key = [&](auto below) {
        int64_t a = kmin, b = kmax;
        while (b - a > 1) {
            const int64_t m = a + (b - a) / 2;
            if (below(atan_death_prob(A, key_float(m)))) a = m; else b = m;
        }
        return a;
    };
    auto never = [&](double p) { return p <= -delta; };
    auto maybe = [&](double p) { return p < 1.0 + delta; };
    if (never(atan_death_prob(A, -INFINITY)) && !never(atan_death_prob(A, INFINITY)))
        A.age_lo = key_float(last_key(never));
    if (maybe(atan_death_prob(A, -INFINITY)) && !maybe(atan_death_prob(A, INFINITY)))
        A.age_hi = key_float(last_key(maybe));
}

// Numerical Recipes' log-gamma, continued fraction and regularised incomplete
// beta function I_x(a, b) (Press et al., Numerical Recipes in C, 2nd ed.,
// 6.1 and 6.4), the functions the reference's utils/bino_tools.cpp uses.
static double nr_lngamma(double xx) {
    static const double c[6] = {76.18009172947146, -86.50532032941677, 24.01409824083091,
                                -1.231739572450155, 0.1208650973866179e-2, -0.5395239384953e-5};
    double y = xx + 1;
    double t = xx + 5.5;
    t -= (xx + 0.5) * std::log(t);
    double ser = 1.000000000190015;
    for (int j = 0; j < 6; j++) {
        ser += c[j] / y;
        y++;
    }
    return -t + std::log(2.5066282746310005 * ser / xx);
}

static double nr_beta_cf(double a, double b, double x) {
    const double tiny = (double)1.0e-30f;
    const double qab = a + b, qap = a + 1.0, qam = a - 1.0;
    double c = 1.0;
    double d = 1.0 - qab * x / qap;
    if (std::fabs(d) < tiny) d = tiny;
    d = 1.0 / d;
    double h = d;
    int m = 1;
    for (; m <= 100; m++) {
        const int m2 = 2 * m;
        double aa = m * (b - m) * x / ((qam + m2) * (a + m2));
        d = 1.0 + aa * d;
        if (std::fabs(d) < tiny) d = tiny;
        c = 1.0 + aa / c;
        if (std::fabs(c) < tiny) c = tiny;
        d = 1.0 / d;
        h *= d * c;
        aa = -(a + m) * (qab + m) * x / ((a + m2) * (qap + m2));
        d = 1.0 + aa * d;
        if (std::fabs(d) < tiny) d = tiny;
        c = 1.0 + aa / c;
        if (std::fabs(c) < tiny) c = tiny;
        d = 1.0 / d;
        const double del = d * c;
        h *= del;
        if (std::fabs(del - 1.0) < 3.0e-7) break;
    }
    return m > 100 ? -1.0 : h;
}

static double nr_beta_inc(double a, double b, double x) {
    if (x < 0.0 || x > 1.0) return -1.0;
    double bt = 0.0;
    if (x != 0.0 && x != 1.0) {
        bt = std::exp(nr_lngamma(a + b) - nr_lngamma(a) - nr_lngamma(b) + a * std::log(x) + b * std::log(1.0 - x));
    }
    if (x < (a + 1.0) / (a + b + 2.0)) return bt * nr_beta_cf(a, b, x) / a;
    return 1.0 - bt * nr_beta_cf(b, a, 1.0 - x) / b;
}

// BinomialDist::buildTable (utils/BinomialDist.cpp:61-89): entry k-1 is
// P(X < k) = 1 - I_p(k, n-k+1) for X ~ Binomial(n, p), k = 1, 2, ... until the
// tail I_p drops to eps (the entry of that k included)
static std::vector<double> binomial_table(double p, int n, double eps) {
    std::vector<double> v;
    int k = 1;
    double tail = nr_beta_inc(k, n - k + 1, p);
    while (tail > eps && k < n && v.size() <= (size_t)kMaxBinomial) {
        v.push_back(tail);
        k++;
        tail = nr_beta_inc(k, n - k + 1, p);
    }
    v.push_back(tail);
    for (double &x : v) x = 1 - x;
    return v;
}

// BinomialDist::getN compares wrandd() = u / 2^32 > L; u / 2^32 > L <=> u > floor(L * 2^32)
static int64_t bino_threshold(double L) {
    const double y = std::floor(L * 4294967296.0);
    if (y >= 4294967296.0) return 4294967296ll;
    if (y < -1.0) return -1ll;
    return (int64_t)y;
}

// Per-action constants and the step flags of an action list given in
// execution order; draw windows are handed out in that order.
int qhg_host_actions(StepConst &P, int n, const int32_t *types, const double (*params)[4], std::string &err) {
    uint32_t w = 0;
    if (P.dense_cell == 0u) P.dense_cell = kDenseCell;
    for (int a = 0; a < n; a++) {
        ActionConst &A = P.act[a];
        const double *p = params[a];
        A.type = types[a];
        A.window = w;
        switch (A.type) {
        case kGetOld:
            P.age_from_birth = 1;
            break;
        case kFertility:
            A.f0 = (float)p[0]; A.f1 = (float)p[1]; A.f2 = (float)p[2];
            if (!P.age_from_birth) P.reads_age = 1;   // reads the age before any GetOld sets it
            break;
        case kRandomPair:
            P.has_pair = 1;
            break;
        case kVerhulst:
        case kVerhulstVarK:
            if (P.n_verhulst >= kMaxVerhulst) {
                err = "more than one Verhulst action";
                return -1;
            }
            A.vslot = P.n_verhulst;
            P.verhulst_act[P.n_verhulst++] = a;
            A.b0 = p[0]; A.d0 = p[1]; A.th = p[2];
            A.th_b0 = p[2] - p[0];
            A.th_d0 = p[2] - p[1];
            A.K = p[3];
            w += 2;
            break;
        case kOldAgeDeath: {
            // OldAgeDeath::execute (actions/OldAgeDeath.cpp:57-60):
            // age > M + wrandr(1 - U*M, 1 + U*M)
            const double M = p[0], U = p[1];
            const double lo = 1 - U * M;
            const double hi = 1 + U * M;
            const double wd = hi - lo;
            A.oad_M = M; A.oad_a = lo; A.oad_w = wd;
            const double g0 = M + (lo + (wd * 0.0) / 4294967296.0);
            const double g1 = M + (lo + (wd * 4294967295.0) / 4294967296.0);
            A.age_lo = float_floor_of(g0);
            A.age_hi = float_floor_of(g1);
            P.age_from_birth = 1;
            w += 1;
            break;
        }
        case kATanDeath:
            // ATanDeath::preLoop (actions/ATanDeath.cpp:41):
            // scale = (pi/2 - EPS) / atan(slope * range)
            A.at_M = p[0];
            A.at_slope = p[2];
            A.at_scale = (kQPi / 2 - kATanEps) / std::atan(p[2] * p[1]);
            atan_death_window(A);
            P.age_from_birth = 1;
            w += 1;
            break;
        case kRandomMove:
        case kWeightedMove:
            A.pthr = host_prob_threshold(p[0]);
            P.has_move = 1;
            if (A.type == kWeightedMove) P.has_wmove = 1;
            w += 2;
            break;
        default:
            err = "unknown action type";
            return -1;
        }
    }
    if (w > 4 * 64) {
        err = "too many draws per agent";
        return -1;
    }
    return 0;
}

// The slots of each cell's move word that WeightedMove may move to (bits
// 24-29): those holding a neighbour that is not ice.  WeightedMove::execute
// registers no move into a cell the grid's Geography marks as ice
// (actions/WeightedMove.cpp:91); ice == nullptr: no Geography, no ice.
void qhg_host_ice_bits(int C, const int32_t *nbr6, const uint8_t *ice, std::vector<uint32_t> &cmove) {
    for (int c = 0; c < C; c++) {
        uint32_t wv = 0;
        for (int j = 0; j < 6; j++) {
            const int d = nbr6[(size_t)c * 6 + j];
            if (d >= 0 && (ice == nullptr || ice[d] == 0)) wv |= 1u << j;
        }
        cmove[c] = (cmove[c] & ~(63u << 24)) | (wv << 24);
    }
}

// Runs f(c0, c1) over [0, n) in contiguous chunks on the host's cores (the
// grid tables of large grids: every cell independent); returns the smallest
// cell at which some chunk reported an error (f returns the failing cell, or
// n when its chunk went through), n if none.
template <class F>
static int parallel_cells(int n, F f) {
    unsigned hw = std::thread::hardware_concurrency();
    const int nt = (int)std::max(1u, std::min(hw == 0u ? 1u : hw, 32u));
    if (n < 65536 || nt == 1) return f(0, n);
    std::vector<int> bad((size_t)nt, n);
    std::vector<std::thread> th;
    const int per = (n + nt - 1) / nt;
    for (int t = 0; t < nt; t++) {
        const int c0 = t * per, c1 = std::min(n, c0 + per);
        if (c0 >= c1) break;
        th.emplace_back([&, t, c0, c1]() { bad[(size_t)t] = f(c0, c1); });
    }
    for (auto &x : th) x.join();
    int b = n;
    for (int v : bad) b = std::min(b, v);
    return b;
}

// Grid tables of one run: rev packs, 3 bits per neighbour slot q, the slot
// of the cell in the neighbour's own list; wthr holds the WeightedMove
// thresholds (SingleEvaluator's cumulated weights, actions/SingleEvaluator.cpp:174-241,
// as integers: dR2 = wrandd()*W[n] < W[j]  <=>  u < T_j); cmove packs per cell
// the neighbour count (bits 0-2), the slots that hold a neighbour (bits 8-13),
// whether all weights are equal (bit 16) and the slots WeightedMove may move
// to (bits 24-29, not ice).  The SingleEvaluator gives an ice cell weight 0
// (actions/SingleEvaluator.cpp:183-202).
int qhg_host_grid_tables(int C, const int32_t *nbr6, const uint8_t *nnbr, const double *K, bool wm,
                         const uint8_t *ice, std::vector<uint32_t> &rev, std::vector<uint64_t> &wthr,
                         std::vector<uint32_t> &cmove, std::string &err) {
    // one pass over the cells on all host cores: reverse slots, move words,
    // each cell's own SingleEvaluator weight (every element is written: the
    // weights need no zero fill)
    rev.resize((size_t)C);
    cmove.resize((size_t)C);
    std::unique_ptr<double[]> W(wm ? new double[(size_t)C * 7] : nullptr);
    // the first failing cell's problem: 1 too many neighbours, 2 index out of
    // range, 3 not symmetric
    std::vector<uint8_t> why((size_t)C, 0u);
    const int bad = parallel_cells(C, [&](int c0, int c1) {
        for (int c = c0; c < c1; c++) {
            if (nnbr[c] > 6) { why[(size_t)c] = 1u; return c; }
            uint32_t rv = 0u, vm = 0u, wv = 0u;
            for (int j = 0; j < 6; j++) {
                const int d = nbr6[(size_t)c * 6 + j];
                if (d >= C || d < -1) { why[(size_t)c] = 2u; return c; }
                if (d >= 0) {
                    vm |= 1u << j;
                    if (ice == nullptr || ice[d] == 0) wv |= 1u << j;
                }
                if (j >= nnbr[c] || d < 0) continue;
                int k = -1;
                for (int q = 0; q < nnbr[d] && q < 6; q++) {
                    if (nbr6[(size_t)d * 6 + q] == c) { k = q; break; }
                }
                if (k < 0) { why[(size_t)c] = 3u; return c; }
                rv |= (uint32_t)k << (3 * j);
            }
            rev[(size_t)c] = rv;
            // neighbour count, slots holding a neighbour, slots a WeightedMove may enter
            cmove[(size_t)c] = (uint32_t)nnbr[c] | (vm << 8) | (wv << 24);
            if (wm) {
                const double dV = K[c];
                W[(size_t)c * 7] = (ice != nullptr && ice[c] != 0) ? 0 : ((dV > 0) ? dV : 0);
            }
        }
        return C;
    });
    if (bad < C) {
        const uint8_t w = why[(size_t)bad];
        err = w == 1u ? "more than 6 neighbours" : (w == 2u ? "neighbour index out of range"
                                                            : "neighbour table is not symmetric");
        return -1;
    }
    if (!wm) {
        wthr.assign((size_t)C * 6, 0);
        return 0;
    }
    parallel_cells(C, [&](int c0, int c1) {
        for (int c = c0; c < c1; c++) {
            double dW = W[(size_t)c * 7];
            for (int i = 0; i < 6; i++) {
                double dCW = 0;
                const int ni = nbr6[(size_t)c * 6 + i];
                if (ni >= 0) dCW = W[(size_t)ni * 7];
                dCW = (dCW > 0) ? dCW : 0;
                dW = dW + dCW;
                W[(size_t)c * 7 + i + 1] = dW;
            }
        }
        return C;
    });
    return qhg_host_move_tables(C, nnbr, W.get(), wthr, cmove, err);
}

// WeightedMove's thresholds from cumulative weights W (C x 7, W[c][0] the
// cell's own, W[c][i+1] = W[c][i] + neighbour i's; WeightedMove::execute,
// actions/WeightedMove.cpp:57-80).  A cell with W[c][0] == W[c][n] draws its
// direction with wrandi (bit 16 of its move word).  Otherwise the agent goes
// to the first j with dR2 = wrandd() * W[c][n] < W[c][j]; dR2 rises with the
// draw u, so "dR2 < W[c][j]" holds exactly for u below T_j, the smallest u
// with dR2 >= W[c][j].  The first j with u < T_j is the number of j whose
// running maximum max(T_0..T_j) is <= u, which is what the device counts
// (j = n always qualifies: dR2 < W[c][n]).  The running maximum makes this
// exact for rows that are not monotone too; it needs W[c][n] > 0 and finite
// weights, which the rows of any cell that is not all-equal must have.
// wthr gets T per cell and slot; cmove's bit 16 is set here, its other bits
// are left as they are.
int qhg_host_move_tables(int C, const uint8_t *nnbr, const double *W, std::vector<uint64_t> &wthr,
                         std::vector<uint32_t> &cmove, std::string &err) {
    // every slot of every cell is written below (the vector keeps its size
    // when a caller filled it already)
    wthr.resize((size_t)C * 6);
    // per failing cell: 1 total weight not positive and finite, 2 a weight not finite
    std::vector<uint8_t> why((size_t)C, 0u);
    const int bad = parallel_cells(C, [&](int c0, int c1) {
        for (int c = c0; c < c1; c++) {
            const int nn = nnbr[c];
            const double *Wc = &W[(size_t)c * 7];
            const double Wn = Wc[nn];
            cmove[c] &= ~(1u << 16);
            if (Wc[0] == Wn) {
                cmove[c] |= 1u << 16;
                for (int j = 0; j < 6; j++) wthr[(size_t)c * 6 + j] = 0;
                continue;
            }
            if (!(Wn > 0.0) || !std::isfinite(Wn)) { why[(size_t)c] = 1u; return c; }
            // wrandd() * W[n] for the draw u: u / 2^32 is exact, so it is u * 2^-32
            auto f = [&](uint64_t u) { return ((double)u * 0x1p-32) * Wn; };
            // where the search starts (the loops below settle u exactly)
            const double guess = 4294967296.0 / Wn;
            uint64_t run = 0;
            for (int j = 0; j < nn; j++) {
                const double x = Wc[j];
                if (!std::isfinite(x)) { why[(size_t)c] = 2u; return c; }
                // smallest u in [0, 2^32] with f(u) >= x  (f(2^32) counts as +inf)
                double g = std::floor(x * guess);
                uint64_t u = (g <= 0) ? 0ull : (g >= 4294967296.0 ? 4294967296ull : (uint64_t)g);
                while (u > 0 && f(u - 1) >= x) u--;
                while (u < 4294967296ull && f(u) < x) u++;
                run = std::max(run, u);
                wthr[(size_t)c * 6 + j] = run;
            }
            // slots without a neighbour: 2^32, a threshold no draw reaches (the
            // device may count over all six slots)
            for (int j = nn; j < 6; j++) wthr[(size_t)c * 6 + j] = 4294967296ull;
        }
        return C;
    });
    if (bad < C) {
        err = "cell " + std::to_string(bad) +
              (why[(size_t)bad] == 1u ? ": total move weight not positive and finite" : ": move weight not finite");
        return -1;
    }
    return 0;
}

extern "C" const char *qhg_gpu_last_error(void) { return g_last_error.c_str(); }

extern "C" const char *qhg_gpu_version(void) { return "qhg_gpu 0.1 (sm_103a)"; }

extern "C" int qhg_gpu_create(const qhg_run_desc *desc, qhg_run **out) {
    if (desc == nullptr || out == nullptr) return fail(QHG_ERR_ARG, "null argument");
    if (desc->n_actions < 0 || desc->n_actions > QHG_MAX_ACTIONS) return fail(QHG_ERR_ARG, "bad n_actions");
    if (desc->genome_size < 0) return fail(QHG_ERR_ARG, "bad genome_size");
    if (desc->genome_size > kMaxGenomeBlocks * 64) return fail(QHG_ERR_ARG, "genome_size above 4096 loci");
    if (desc->genome_size > 0 && desc->num_crossover != QHG_CROSSOVER_POISSON1 &&
        (desc->num_crossover < 0 || desc->num_crossover > kMaxFixedCrossover)) {
        return fail(QHG_ERR_ARG, "num_crossover must be QHG_CROSSOVER_POISSON1 or in 0..30");
    }
    if (desc->genome_size > 0 && !(desc->mutation_rate >= 0.0 && desc->mutation_rate < 1.0)) {
        return fail(QHG_ERR_ARG, "mutation_rate must be in [0, 1)");
    }
    int ndev = 0;
    CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (desc->device < 0 || desc->device >= ndev) return fail(QHG_ERR_ARG, "bad device ordinal");
    CUDA_TRY(cudaSetDevice(desc->device));
    qhg_run *r = new qhg_run();
    r->desc = *desc;
    StepConst &P = r->P;
    memset(&P, 0, sizeof(P));
    P.seed = desc->seed;
    philox_round_keys(P.seed, P.rkey);
    P.n_act = desc->n_actions;
    P.log_births = (desc->flags & QHG_FLAG_LOG_BIRTHS) ? 1 : 0;
    {
        std::string err;
        if (qhg_host_actions(P, desc->n_actions, desc->action_type, desc->action_param, err) != 0) {
            delete r;
            return fail(QHG_ERR_ARG, err);
        }
    }
    if (desc->genome_size > 0) {
        P.genome_size = desc->genome_size;
        P.genome_words = 2 * ((desc->genome_size + 63) / 64);
        P.num_crossover = desc->num_crossover;
        P.has_mutation = desc->mutation_rate > 0.0 ? 1 : 0;
        if (P.has_mutation) {
            std::vector<double> tab = binomial_table(desc->mutation_rate, 2 * desc->genome_size, 1e-6);
            if ((int)tab.size() > kMaxBinomial) {
                delete r;
                return fail(QHG_ERR_ARG, "mutation rate too high: more than 64 mutation counts in the table");
            }
            P.n_binomial = (int32_t)tab.size();
            for (size_t i = 0; i < tab.size(); i++) P.bino[i] = bino_threshold(tab[i]);
        }
    }
    P.program = qhg_match_program(desc->action_type, desc->n_actions);
    // a specialised program takes its draws at fixed windows: keep it only if
    // the windows handed out match them
    for (int a = 0; P.program > 0 && a < desc->n_actions; a++) {
        if (P.act[a].window != qhg_program_window(P.program, a)) P.program = 0;
    }
    cudaError_t e = cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&r->d_rs, sizeof(RunState));
    if (e == cudaSuccess) e = cudaMallocHost(&r->h_rs, sizeof(RunState));
    if (e != cudaSuccess) {
        if (r->stream) cudaStreamDestroy(r->stream);
        cudaFree(r->d_rs);
        delete r;
        return fail(QHG_ERR_CUDA, std::string("create: ") + cudaGetErrorString(e));
    }
    memset(r->h_rs, 0, sizeof(RunState));
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, desc->device);
    // persistent grids of the tile kernels: as many CTAs as fit at once
    int ca = 1, cs = 1;
    qhg_tile_ctas_per_sm(&ca, &cs);
    r->shape.actions_grid = std::max(1, nsm) * ca;
    r->shape.scatter_grid = std::max(1, nsm) * cs;
    r->shape.big_grid = std::max(1, nsm);
    *out = r;
    return QHG_OK;
}

static int ms_reset(qhg_run *r);
static void ms_free(qhg_run *r);

static const uint8_t *ice_ptr(const qhg_run *r) { return r->h_ice.empty() ? nullptr : r->h_ice.data(); }

// The grid's neighbour table, neighbour counts and K as host copies, for the
// updates between steps that rebuild tables on the host (fetched from the
// device on first use: the upload keeps none)
static int host_grid(qhg_run *r) {
    if (!r->h_nbr.empty()) return QHG_OK;
    const size_t C = (size_t)r->C;
    r->h_nbr.resize(C * 6);
    r->h_nnbr.resize(C);
    r->h_K.resize(C);
    CUDA_TRY(cudaMemcpyAsync(r->h_nbr.data(), r->d_nbr, C * 6 * sizeof(int32_t), cudaMemcpyDeviceToHost, r->stream));
    CUDA_TRY(cudaMemcpyAsync(r->h_nnbr.data(), r->d_nnbr, C, cudaMemcpyDeviceToHost, r->stream));
    CUDA_TRY(cudaMemcpyAsync(r->h_K.data(), r->d_K, C * sizeof(double), cudaMemcpyDeviceToHost, r->stream));
    CUDA_TRY(cudaStreamSynchronize(r->stream));
    return QHG_OK;
}

extern "C" int qhg_gpu_upload_grid(qhg_run *r, const int32_t *nbr6, const uint8_t *nnbr, const double *K,
                                   int32_t num_cells) {
    if (r == nullptr || nbr6 == nullptr || nnbr == nullptr || K == nullptr || num_cells <= 0) {
        return fail(QHG_ERR_ARG, "bad grid arguments");
    }
    CUDA_TRY(cudaSetDevice(r->desc.device));
    const int C = num_cells;
    cudaStream_t st = r->stream;
    // the grid tables are built on the device in new buffers; a grid that is
    // rejected leaves the run as it was
    int32_t *n_nbr = nullptr;
    uint8_t *n_nnbr = nullptr;
    double *n_K = nullptr, *tW = nullptr;
    uint32_t *n_rev = nullptr, *n_cmove = nullptr;
    uint64_t *n_wthr = nullptr;
    unsigned long long *d_bad = nullptr;
    auto release = [&]() {
        cudaFree(n_nbr); cudaFree(n_nnbr); cudaFree(n_K); cudaFree(n_rev); cudaFree(n_cmove); cudaFree(n_wthr);
        cudaFree(tW); cudaFree(d_bad);
    };
    const bool wm = r->P.has_wmove != 0;
    cudaError_t e = cudaMalloc(&n_nbr, (size_t)C * 6 * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&n_nnbr, (size_t)C);
    if (e == cudaSuccess) e = cudaMalloc(&n_K, (size_t)C * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&n_rev, (size_t)C * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&n_cmove, (size_t)C * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&n_wthr, (size_t)C * 6 * sizeof(uint64_t));
    if (e == cudaSuccess && wm) e = cudaMalloc(&tW, (size_t)C * 7 * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&d_bad, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemcpyAsync(n_nbr, nbr6, (size_t)C * 6 * sizeof(int32_t), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(n_nnbr, nnbr, (size_t)C, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(n_K, K, (size_t)C * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_bad, 0xff, sizeof(unsigned long long), st);
    if (e == cudaSuccess && !wm) e = cudaMemsetAsync(n_wthr, 0, (size_t)C * 6 * sizeof(uint64_t), st);
    if (e != cudaSuccess) {
        release();
        return fail(e == cudaErrorMemoryAllocation ? QHG_ERR_NOMEM : QHG_ERR_CUDA, cudaGetErrorString(e));
    }
    unsigned long long bad = ~0ull;
    for (int pass = 0; pass < (wm ? 2 : 1); pass++) {
        // the weights' pass reads neighbours' rows: only over a valid table
        int le = qhg_launch_grid_tables(C, n_nbr, n_nnbr, n_K, wm ? 1 : 0, n_rev, n_cmove, tW, n_wthr, d_bad, pass, st);
        cudaError_t ce = le == 0 ? cudaMemcpyAsync(&bad, d_bad, sizeof(bad), cudaMemcpyDeviceToHost, st) : (cudaError_t)le;
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
        if (ce != cudaSuccess) {
            release();
            return fail(QHG_ERR_CUDA, std::string("grid tables: ") + cudaGetErrorString(ce));
        }
        if (bad != ~0ull) {
            release();
            const unsigned long long cell = bad >> 8;
            switch ((int)(bad & 0xffull)) {
            case 1: return fail(QHG_ERR_ARG, "more than 6 neighbours");
            case 2: return fail(QHG_ERR_ARG, "neighbour index out of range");
            case 3: return fail(QHG_ERR_ARG, "neighbour table is not symmetric");
            case 4: return fail(QHG_ERR_ARG, "cell " + std::to_string(cell) + ": total move weight not positive and finite");
            default: return fail(QHG_ERR_ARG, "cell " + std::to_string(cell) + ": move weight not finite");
            }
        }
    }
    cudaFree(tW);
    tW = nullptr;
    cudaFree(d_bad);
    d_bad = nullptr;
    cudaFree(r->d_nbr); cudaFree(r->d_nnbr); cudaFree(r->d_rev); cudaFree(r->d_K); cudaFree(r->d_vthr[0]); cudaFree(r->d_vthr[1]);
    cudaFree(r->d_wthr); cudaFree(r->d_cmove); cudaFree(r->d_occ);
    cudaFree(r->d_clsc); cudaFree(r->d_sbase); cudaFree(r->d_bbase); cudaFree(r->d_bidb);
    cudaFree(r->d_obase); cudaFree(r->d_tflag); cudaFree(r->d_tagg); cudaFree(r->d_tincl);
    ms_free(r);
    r->d_nbr = n_nbr;
    r->d_nnbr = n_nnbr;
    r->d_K = n_K;
    r->d_rev = n_rev;
    r->d_cmove = n_cmove;
    r->d_wthr = n_wthr;
    r->d_vthr[0] = r->d_vthr[1] = nullptr;
    r->d_occ = nullptr;
    r->grid_ok = false;
    r->agents_ok = false;
    drop_graphs(r);
    const int ntiles = (C + kScanTile - 1) / kScanTile;
    CUDA_TRY(cudaMalloc(&r->d_vthr[0], (size_t)C * sizeof(ulonglong2)));
    CUDA_TRY(cudaMalloc(&r->d_vthr[1], (size_t)C * sizeof(ulonglong2)));
    if (r->desc.flags & QHG_FLAG_TRACK_OCCUPANCY) {
        CUDA_TRY(cudaMalloc(&r->d_occ, (size_t)C * sizeof(int32_t)));
        CUDA_TRY(cudaMemsetAsync(r->d_occ, 0xff, (size_t)C * sizeof(int32_t), st));
    }
    CUDA_TRY(cudaMalloc(&r->d_clsc, (size_t)C * kCls * sizeof(uint32_t)));
    CUDA_TRY(cudaMalloc(&r->d_sbase, (size_t)C * sizeof(uint32_t)));
    CUDA_TRY(cudaMalloc(&r->d_bbase, (size_t)C * sizeof(uint32_t)));
    CUDA_TRY(cudaMalloc(&r->d_bidb, (size_t)C * sizeof(uint32_t)));
    CUDA_TRY(cudaMalloc(&r->d_obase, (size_t)C * 6 * sizeof(uint32_t)));
    CUDA_TRY(cudaMalloc(&r->d_tflag, (size_t)ntiles * sizeof(uint32_t)));
    CUDA_TRY(cudaMalloc(&r->d_tagg, (size_t)ntiles * sizeof(uint4)));
    CUDA_TRY(cudaMalloc(&r->d_tincl, (size_t)ntiles * sizeof(uint4)));
    CUDA_TRY(cudaMemsetAsync(r->d_clsc, 0, (size_t)C * kCls * sizeof(uint32_t), st));
    CUDA_TRY(cudaMemsetAsync(r->d_tflag, 0, (size_t)ntiles * sizeof(uint32_t), st));
    CUDA_TRY(cudaStreamSynchronize(st));
    // host copies of the grid are fetched when an update needs them
    r->h_nbr.clear();
    r->h_nnbr.clear();
    r->h_K.clear();
    r->w_given = false;
    r->h_ice.clear();
    r->C = C;
    r->P.num_cells = C;
    r->grid_ok = true;
    return QHG_OK;
}

static int alloc_agents(qhg_run *r, uint32_t cap) {
    free_agents(r);
    const int C = r->C;
    for (int p = 0; p < 2; p++) {
        CUDA_TRY(cudaMalloc(&r->d_id[p], (size_t)cap * sizeof(int64_t) + kColumnPad));
        CUDA_TRY(cudaMalloc(&r->d_birth[p], (size_t)cap * sizeof(float) + kColumnPad));
        CUDA_TRY(cudaMalloc(&r->d_age[p], (size_t)cap * sizeof(float) + kColumnPad));
        CUDA_TRY(cudaMalloc(&r->d_lastb[p], (size_t)cap * sizeof(float) + kColumnPad));
        CUDA_TRY(cudaMalloc(&r->d_meta[p], (size_t)cap + kColumnPad));
        CUDA_TRY(cudaMalloc(&r->d_ne[p], (size_t)C * sizeof(uint32_t)));
        CUDA_TRY(cudaMalloc(&r->d_necm[p], (size_t)C * sizeof(uint32_t)));
        CUDA_TRY(cudaMalloc(&r->d_nes[p], (size_t)(C + 1) * sizeof(uint32_t)));
        CUDA_TRY(cudaMalloc(&r->d_tf[p], ((size_t)cap / kTileAgents + 2) * sizeof(uint32_t)));
    }
    CUDA_TRY(cudaMalloc(&r->d_outc, (size_t)cap * sizeof(uint32_t) + kColumnPad));
    CUDA_TRY(cudaMalloc(&r->d_father, (size_t)cap * sizeof(int32_t) + kColumnPad));   // staged by the cell scatter
    CUDA_TRY(cudaMalloc(&r->d_brank, (size_t)cap * sizeof(uint16_t)));
    if (r->P.log_births) {
        r->blog_cap = std::max<uint64_t>(1u << 20, (uint64_t)cap * 4);
        CUDA_TRY(cudaMalloc(&r->d_blog, r->blog_cap * 3 * sizeof(int64_t)));
    } else {
        r->blog_cap = 0;
    }
    if (r->P.genome_words > 0) {
        // slots in use during a step: the live agents plus the step's births
        // (at most one per live female), so 2 * capacity never runs out
        const uint64_t g = std::min<uint64_t>((uint64_t)cap * 2, 0x7fffffffull);
        for (int p = 0; p < 2; p++) {
            CUDA_TRY(cudaMalloc(&r->d_gslot[p], (size_t)cap * sizeof(int32_t) + kColumnPad));
            CUDA_TRY(cudaMalloc(&r->d_free[p], (size_t)g * sizeof(uint32_t)));
        }
        CUDA_TRY(cudaMalloc(&r->d_genome, (size_t)g * r->P.genome_words * sizeof(uint64_t)));
        CUDA_TRY(cudaMalloc(&r->d_brec, (size_t)cap * 5 * sizeof(uint32_t)));
        r->gcap = (uint32_t)g;
        r->P.genome_capacity = (uint32_t)g;
    }
    r->cap = cap;
    r->P.capacity = cap;
    return QHG_OK;
}

static StepBuffers make_buffers(qhg_run *r, int cur);

// Uploads are sorted by cell on the device (k_upload_count, k_cell_scan,
// k_upload_place): the caller's columns are copied as they are, with the
// next table's buffers as staging.
extern "C" int qhg_gpu_upload_agents(qhg_run *r, const qhg_agents_soa *a, int64_t n, int32_t first_step) {
    if (r == nullptr || a == nullptr || n < 0) return fail(QHG_ERR_ARG, "bad agent arguments");
    if (!r->grid_ok) return fail(QHG_ERR_STATE, "upload the grid before the agents");
    if (n > 0 && (a->id == nullptr || a->cell == nullptr || a->birth == nullptr || a->age == nullptr ||
                  a->last_birth == nullptr || a->gender == nullptr || a->state == nullptr)) {
        return fail(QHG_ERR_ARG, "null agent column");
    }
    if (n > 0 && r->P.genome_words > 0 && a->genome == nullptr) return fail(QHG_ERR_ARG, "null genome column");
    if (first_step < 0) return fail(QHG_ERR_ARG, "negative first step");
    CUDA_TRY(cudaSetDevice(r->desc.device));
    const int C = r->C;
    // the capacity also holds the staged input rows (dead ones included)
    uint64_t want = r->desc.agent_capacity > 0 ? (uint64_t)r->desc.agent_capacity : (uint64_t)n * 4 + 65536;
    if (want < (uint64_t)n) want = (uint64_t)n;
    if (want > 0x7fffffffull) return fail(QHG_ERR_CAPACITY, "agent capacity above 2^31-1");
    drop_graphs(r);
    r->agents_ok = false;
    if (r->cap != (uint32_t)want || r->d_id[0] == nullptr) {
        int rc = alloc_agents(r, (uint32_t)want);
        if (rc != QHG_OK) return rc;
    }
    cudaStream_t st = r->stream;
    // staging: table 1's columns, the father column for cells, the birth-rank
    // column for gender and state
    int32_t *s_cell = r->d_father;
    uint8_t *s_gender = reinterpret_cast<uint8_t *>(r->d_brank);
    uint8_t *s_state = s_gender + r->cap;
    if (n > 0) {
        CUDA_TRY(cudaMemcpyAsync(r->d_id[1], a->id, n * sizeof(int64_t), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(r->d_birth[1], a->birth, n * sizeof(float), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(r->d_age[1], a->age, n * sizeof(float), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(r->d_lastb[1], a->last_birth, n * sizeof(float), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(s_cell, a->cell, n * sizeof(int32_t), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(s_gender, a->gender, n, cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(s_state, a->state, n, cudaMemcpyHostToDevice, st));
        if (r->P.genome_words > 0) {
            // genome slot = input row
            CUDA_TRY(cudaMemcpyAsync(r->d_genome, a->genome, (size_t)n * r->P.genome_words * sizeof(uint64_t),
                                     cudaMemcpyHostToDevice, st));
        }
    }
    memset(r->h_rs, 0, sizeof(RunState));
    r->h_rs->step = first_step;
    r->h_rs->next_id = -1;   // the largest ID, by the count kernel
    CUDA_TRY(cudaMemcpyAsync(r->d_rs, r->h_rs, sizeof(RunState), cudaMemcpyHostToDevice, st));
    const int ntiles = (C + kScanTile - 1) / kScanTile;
    CUDA_TRY(cudaMemsetAsync(r->d_tflag, 0, (size_t)ntiles * sizeof(uint32_t), st));
    CUDA_TRY(cudaMemsetAsync(r->d_clsc, 0, (size_t)C * kCls * sizeof(uint32_t), st));
    // the scan writes the lists of the table in buffer 0 ("next" of buffer 1)
    StepBuffers B = make_buffers(r, 1);
    int le = qhg_launch_upload(&r->P, r->d_rs, &B, s_cell, s_gender, s_state, r->d_id[1], r->d_birth[1],
                               r->d_age[1], r->d_lastb[1], n, r->P.genome_words > 0 ? r->d_gslot[0] : nullptr, st);
    if (le != 0) return fail(QHG_ERR_CUDA, std::string("upload: ") + cudaGetErrorString((cudaError_t)le));
    CUDA_TRY(cudaMemcpyAsync(r->h_rs, r->d_rs, sizeof(RunState), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    r->launched = 0;
    RunState *h = r->h_rs;
    if (h->error != 0u) {
        const uint32_t code = h->error;
        memset(h, 0, sizeof(RunState));
        CUDA_TRY(cudaMemcpyAsync(r->d_rs, h, sizeof(RunState), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemsetAsync(r->d_clsc, 0, (size_t)C * kCls * sizeof(uint32_t), st));
        CUDA_TRY(cudaStreamSynchronize(st));
        if (code == kErrBadCell) return fail(QHG_ERR_ARG, "agent cell out of range");
        if (code == kErrCellTooLarge) return fail(QHG_ERR_CELL_TOO_LARGE, "a cell holds more than QHG_MAX_CELL_AGENTS agents");
        if (code == kErrCapacity) return fail(QHG_ERR_CAPACITY, "agents exceed the capacity");
        return fail(QHG_ERR_DEVICE, "upload failed on the device");
    }
    // commit the uploaded table as the current one
    const int64_t maxid = h->next_id;
    const uint32_t live = h->new_n_agents;
    const uint32_t nne = h->new_n_nonempty;
    const uint32_t form = step_form(h->max_cell, live, nne, r->P.dense_cell);
    memset(h, 0, sizeof(RunState));
    h->step = first_step;
    h->n_agents = live;
    h->n_nonempty = nne;
    h->next_id = maxid + 1;
    h->hwm = (uint32_t)n;
    h->form = form;
    h->form_next = form;
    CUDA_TRY(cudaMemcpyAsync(r->d_rs, h, sizeof(RunState), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemsetAsync(r->d_tflag, 0, (size_t)ntiles * sizeof(uint32_t), st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (r->d_occ != nullptr) {
        // the uploaded table's cells are occupied at its step
        CUDA_TRY(cudaMemsetAsync(r->d_occ, 0xff, (size_t)C * sizeof(int32_t), st));
        int le2 = qhg_launch_occupancy(r->d_rs, r->d_ne[0], r->d_occ, r->shape.scatter_grid, st);
        if (le2 != 0) return fail(QHG_ERR_CUDA, std::string("occupancy: ") + cudaGetErrorString((cudaError_t)le2));
        CUDA_TRY(cudaStreamSynchronize(st));
    }
    r->cur = 0;
    r->upload_step = first_step;
    r->upload_max_id = maxid;
    r->agents_ok = true;
    if (r->ms_mode >= 0) return ms_reset(r);
    return QHG_OK;
}

static int pull_state(qhg_run *r);

static StepBuffers make_buffers(qhg_run *r, int cur) {
    const int nx = cur ^ 1;
    StepBuffers B;
    B.nonempty = r->d_ne[cur]; B.ne_start = r->d_nes[cur]; B.tile_first = r->d_tf[cur];
    B.id = r->d_id[cur]; B.birth = r->d_birth[cur]; B.age = r->d_age[cur]; B.lastb = r->d_lastb[cur];
    B.meta = r->d_meta[cur];
    B.nonempty2 = r->d_ne[nx]; B.ne_start2 = r->d_nes[nx]; B.tile_first2 = r->d_tf[nx];
    B.id2 = r->d_id[nx]; B.birth2 = r->d_birth[nx]; B.age2 = r->d_age[nx]; B.lastb2 = r->d_lastb[nx];
    B.meta2 = r->d_meta[nx];
    B.nbr = r->d_nbr; B.nnbr = r->d_nnbr; B.rev = r->d_rev; B.K = r->d_K; B.vthr = r->d_vthr[cur]; B.vthr2 = r->d_vthr[nx]; B.wthr = r->d_wthr;
    B.cmove = r->d_cmove; B.necm = r->d_necm[cur]; B.necm2 = r->d_necm[nx];
    B.occ = r->d_occ;
    B.ms_mode = r->ms_mode;
    B.ms_hops = r->d_ms_hops; B.ms_dist = r->d_ms_dist; B.ms_time = r->d_ms_time;
    B.ms_chops = r->d_ms_chops; B.ms_cdist = r->d_ms_cdist; B.ms_ckey = r->d_ms_ckey; B.ms_D = r->d_ms_D;
    B.outc = r->d_outc; B.father = r->d_father; B.brank = r->d_brank; B.clsc = r->d_clsc;
    B.sbase = r->d_sbase; B.bbase = r->d_bbase; B.bidbase = r->d_bidb; B.obase = r->d_obase;
    B.tile_flag = r->d_tflag; B.tile_agg = r->d_tagg; B.tile_incl = r->d_tincl;
    B.blog = r->d_blog; B.blog_cap = r->blog_cap;
    B.gslot = r->d_gslot[cur]; B.gslot2 = r->d_gslot[nx];
    B.freelist = r->d_free[cur]; B.freelist2 = r->d_free[nx];
    B.genome = r->d_genome; B.brec = r->d_brec;
    return B;
}

static int build_graph(qhg_run *r, int cur) {
    StepBuffers B = make_buffers(r, cur);
    cudaGraph_t g = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(r->stream, cudaStreamCaptureModeThreadLocal));
    int le = qhg_launch_step(&r->P, r->d_rs, &B, nullptr, &r->shape, r->stream);
    cudaError_t ee = cudaStreamEndCapture(r->stream, &g);
    if (le != 0 || ee != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return fail(QHG_ERR_CUDA, std::string("graph capture failed: ") +
                                      cudaGetErrorString(le != 0 ? (cudaError_t)le : ee));
    }
    cudaError_t ie = cudaGraphInstantiate(&r->graph[cur], g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) return fail(QHG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
    return QHG_OK;
}

extern "C" int qhg_gpu_step(qhg_run *r, int32_t nsteps) {
    if (r == nullptr || nsteps < 0) return fail(QHG_ERR_ARG, "bad step arguments");
    if (!r->grid_ok || !r->agents_ok) return fail(QHG_ERR_STATE, "upload grid and agents first");
    CUDA_TRY(cudaSetDevice(r->desc.device));
    for (int32_t s = 0; s < nsteps; s++) {
        if (r->graph[r->cur] == nullptr) {
            int rc = build_graph(r, r->cur);
            if (rc != QHG_OK) return rc;
        }
        CUDA_TRY(cudaGraphLaunch(r->graph[r->cur], r->stream));
        r->cur ^= 1;
        r->launched++;
    }
    return QHG_OK;
}

extern "C" int qhg_gpu_step_timed(qhg_run *r, int32_t nsteps, float *elapsed_ms) {
    if (r == nullptr || elapsed_ms == nullptr) return fail(QHG_ERR_ARG, "null argument");
    CUDA_TRY(cudaSetDevice(r->desc.device));
    if (r->ev[0] == nullptr) {
        for (int i = 0; i < 5; i++) CUDA_TRY(cudaEventCreate(&r->ev[i]));
    }
    CUDA_TRY(cudaEventRecord(r->ev[0], r->stream));
    int rc = qhg_gpu_step(r, nsteps);
    if (rc != QHG_OK) return rc;
    CUDA_TRY(cudaEventRecord(r->ev[1], r->stream));
    CUDA_TRY(cudaEventSynchronize(r->ev[1]));
    CUDA_TRY(cudaEventElapsedTime(elapsed_ms, r->ev[0], r->ev[1]));
    return pull_state(r);
}

extern "C" int qhg_gpu_step_profiled(qhg_run *r, int32_t nsteps, float *kernel_ms) {
    if (r == nullptr || nsteps < 0 || (nsteps > 0 && kernel_ms == nullptr)) return fail(QHG_ERR_ARG, "bad step arguments");
    if (!r->grid_ok || !r->agents_ok) return fail(QHG_ERR_STATE, "upload grid and agents first");
    CUDA_TRY(cudaSetDevice(r->desc.device));
    if (r->ev[0] == nullptr) {
        for (int i = 0; i < 5; i++) CUDA_TRY(cudaEventCreate(&r->ev[i]));
    }
    for (int32_t s = 0; s < nsteps; s++) {
        StepBuffers B = make_buffers(r, r->cur);
        int le = qhg_launch_step_timed(&r->P, r->d_rs, &B, nullptr, &r->shape, r->stream, r->ev);
        if (le != 0) return fail(QHG_ERR_CUDA, std::string("launch: ") + cudaGetErrorString((cudaError_t)le));
        const bool gen = r->P.genome_words > 0;
        CUDA_TRY(cudaEventSynchronize(r->ev[gen ? 4 : 3]));
        for (int k = 0; k < 4; k++) {
            float ms = 0.0f;
            if (k < 3 || gen) CUDA_TRY(cudaEventElapsedTime(&ms, r->ev[k], r->ev[k + 1]));
            kernel_ms[s * 4 + k] = ms;
        }
        r->cur ^= 1;
        r->launched++;
    }
    return QHG_OK;
}

// reads the run state; on a device-side error the run keeps the last
// committed step and its counters are reset so that stepping can resume
static int pull_state(qhg_run *r) {
    CUDA_TRY(cudaMemcpyAsync(r->h_rs, r->d_rs, sizeof(RunState), cudaMemcpyDeviceToHost, r->stream));
    CUDA_TRY(cudaStreamSynchronize(r->stream));
    r->launched = 0;
    r->cur = (int)((uint32_t)(r->h_rs->step - r->upload_step) & 1u);
    if (r->h_rs->error != 0u) {
        const uint32_t code = r->h_rs->error, info = r->h_rs->error_info;
        r->h_rs->error = 0u;
        r->h_rs->error_info = 0u;
        r->h_rs->scan_tiles_started = 0u;
        r->h_rs->scatter_ctas_done = 0u;
        r->h_rs->action_tiles = 0u;
        r->h_rs->scatter_tiles = 0u;
        r->h_rs->dead_count = 0u;
        r->h_rs->max_cell = 0u;
        r->h_rs->stall_tile = 0u;
        // the failed step's partial statistics would be counted again on retry
        unsigned long long *st = r->h_rs->stats[(uint32_t)r->h_rs->step % kStatsRing];
        st[0] = st[1] = st[2] = st[3] = 0ull;
        CUDA_TRY(cudaMemcpyAsync(r->d_rs, r->h_rs, sizeof(RunState), cudaMemcpyHostToDevice, r->stream));
        const int ntiles = (r->C + kScanTile - 1) / kScanTile;
        CUDA_TRY(cudaMemsetAsync(r->d_tflag, 0, (size_t)ntiles * sizeof(uint32_t), r->stream));
        CUDA_TRY(cudaMemsetAsync(r->d_clsc, 0, (size_t)r->C * kCls * sizeof(uint32_t), r->stream));
        CUDA_TRY(cudaStreamSynchronize(r->stream));
        char buf[160];
        switch (code) {
        case kErrCellTooLarge:
            snprintf(buf, sizeof(buf), "cell %u would hold more than %d agents (step %d kept)", info, kMaxCellBig, r->h_rs->step);
            return fail(QHG_ERR_CELL_TOO_LARGE, buf);
        case kErrCapacity:
            snprintf(buf, sizeof(buf), "%u agents exceed the capacity %u (step %d kept)", info, r->cap, r->h_rs->step);
            return fail(QHG_ERR_CAPACITY, buf);
        case kErrTimeout:
            snprintf(buf, sizeof(buf), "cell scan look-back gave up at tile %u (step %d kept)", info, r->h_rs->step);
            return fail(QHG_ERR_TIMEOUT, buf);
        default:
            snprintf(buf, sizeof(buf), "device error %u/%u (step %d kept)", code, info, r->h_rs->step);
            return fail(QHG_ERR_DEVICE, buf);
        }
    }
    return QHG_OK;
}

extern "C" int qhg_gpu_sync(qhg_run *r) {
    if (r == nullptr) return fail(QHG_ERR_ARG, "null run");
    CUDA_TRY(cudaSetDevice(r->desc.device));
    return pull_state(r);
}

// The current table's per-cell constants after K or the move weights changed
// (nothing to do before agents are uploaded: the upload derives them).
static int refresh_cells(qhg_run *r) {
    if (!r->agents_ok || r->h_rs->n_nonempty == 0u) {
        CUDA_TRY(cudaStreamSynchronize(r->stream));
        return QHG_OK;
    }
    const int cur = r->cur;
    const int grid = (int)std::min<uint32_t>((r->h_rs->n_nonempty + 255u) / 256u, 4096u);
    const int le = qhg_launch_refresh_cells(&r->P, r->d_rs, r->d_ne[cur], r->d_nes[cur], r->d_K, r->d_cmove,
                                            r->d_vthr[cur], r->d_necm[cur], grid, r->stream);
    if (le != 0) return fail(QHG_ERR_CUDA, std::string("launch: ") + cudaGetErrorString((cudaError_t)le));
    CUDA_TRY(cudaStreamSynchronize(r->stream));
    return QHG_OK;
}

extern "C" int qhg_gpu_set_capacity(qhg_run *r, const double *K) {
    if (r == nullptr || K == nullptr) return fail(QHG_ERR_ARG, "null argument");
    if (!r->grid_ok) return fail(QHG_ERR_STATE, "upload the grid first");
    CUDA_TRY(cudaSetDevice(r->desc.device));
    {
        const int hg = host_grid(r);   // the grid's host copies (fetched once)
        if (hg != QHG_OK) return hg;
    }
    const int C = r->C;
    // weights that follow K are derived again, as an always-updating
    // SingleEvaluator over K does at the next initialize
    const bool tables = r->P.has_wmove && !r->w_given;
    std::vector<uint32_t> rev, cmove;
    std::vector<uint64_t> wthr;
    if (tables) {
        std::string err;
        if (qhg_host_grid_tables(C, r->h_nbr.data(), r->h_nnbr.data(), K, true, ice_ptr(r), rev, wthr, cmove, err) != 0) {
            return fail(QHG_ERR_ARG, err);
        }
    }
    int rc = pull_state(r);   // the run's steps so far are done (or their error is reported)
    if (rc != QHG_OK) return rc;
    CUDA_TRY(cudaMemcpyAsync(r->d_K, K, (size_t)C * sizeof(double), cudaMemcpyHostToDevice, r->stream));
    if (tables) {
        CUDA_TRY(cudaMemcpyAsync(r->d_wthr, wthr.data(), (size_t)C * 6 * sizeof(uint64_t), cudaMemcpyHostToDevice,
                                 r->stream));
        CUDA_TRY(cudaMemcpyAsync(r->d_cmove, cmove.data(), (size_t)C * sizeof(uint32_t), cudaMemcpyHostToDevice,
                                 r->stream));
    }
    r->h_K.assign(K, K + C);
    return refresh_cells(r);
}

extern "C" int qhg_gpu_set_move_weights(qhg_run *r, const double *cumw7) {
    if (r == nullptr || cumw7 == nullptr) return fail(QHG_ERR_ARG, "null argument");
    if (!r->grid_ok) return fail(QHG_ERR_STATE, "upload the grid first");
    CUDA_TRY(cudaSetDevice(r->desc.device));
    {
        const int hg = host_grid(r);   // the grid's host copies (fetched once)
        if (hg != QHG_OK) return hg;
    }
    const int C = r->C;
    std::vector<uint32_t> rev, cmove;
    std::vector<uint64_t> wthr;
    {
        std::string err;
        // the neighbour bits of the move words, then the weights' thresholds
        if (qhg_host_grid_tables(C, r->h_nbr.data(), r->h_nnbr.data(), r->h_K.data(), false, ice_ptr(r), rev, wthr, cmove,
                                 err) != 0 ||
            qhg_host_move_tables(C, r->h_nnbr.data(), cumw7, wthr, cmove, err) != 0) {
            return fail(QHG_ERR_ARG, err);
        }
    }
    int rc = pull_state(r);
    if (rc != QHG_OK) return rc;
    CUDA_TRY(cudaMemcpyAsync(r->d_wthr, wthr.data(), (size_t)C * 6 * sizeof(uint64_t), cudaMemcpyHostToDevice,
                             r->stream));
    CUDA_TRY(cudaMemcpyAsync(r->d_cmove, cmove.data(), (size_t)C * sizeof(uint32_t), cudaMemcpyHostToDevice,
                             r->stream));
    r->w_given = true;
    return refresh_cells(r);
}

extern "C" int qhg_gpu_set_ice(qhg_run *r, const uint8_t *ice) {
    if (r == nullptr) return fail(QHG_ERR_ARG, "null run");
    if (!r->grid_ok) return fail(QHG_ERR_STATE, "upload the grid first");
    CUDA_TRY(cudaSetDevice(r->desc.device));
    {
        const int hg = host_grid(r);   // the grid's host copies (fetched once)
        if (hg != QHG_OK) return hg;
    }
    const int C = r->C;
    std::vector<uint8_t> flags;
    if (ice != nullptr) {
        flags.resize((size_t)C);
        for (int c = 0; c < C; c++) flags[(size_t)c] = ice[c] != 0 ? 1u : 0u;
    }
    const uint8_t *fp = flags.empty() ? nullptr : flags.data();
    // the move words' WeightedMove slots, and the weights when they follow K
    // (the SingleEvaluator gives ice cells weight 0); given weights stay
    std::vector<uint32_t> rev, cmove;
    std::vector<uint64_t> wthr;
    const bool tables = r->P.has_wmove && !r->w_given;
    {
        std::string err;
        if (qhg_host_grid_tables(C, r->h_nbr.data(), r->h_nnbr.data(), r->h_K.data(), tables, fp, rev, wthr, cmove,
                                 err) != 0) {
            return fail(QHG_ERR_ARG, err);
        }
    }
    int rc = pull_state(r);
    if (rc != QHG_OK) return rc;
    if (tables) {
        CUDA_TRY(cudaMemcpyAsync(r->d_wthr, wthr.data(), (size_t)C * 6 * sizeof(uint64_t), cudaMemcpyHostToDevice,
                                 r->stream));
        CUDA_TRY(cudaMemcpyAsync(r->d_cmove, cmove.data(), (size_t)C * sizeof(uint32_t), cudaMemcpyHostToDevice,
                                 r->stream));
    } else {
        // keep the words' other bits (the given weights' all-equal flags)
        std::vector<uint32_t> cur((size_t)C);
        CUDA_TRY(cudaMemcpyAsync(cur.data(), r->d_cmove, (size_t)C * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                 r->stream));
        CUDA_TRY(cudaStreamSynchronize(r->stream));
        qhg_host_ice_bits(C, r->h_nbr.data(), fp, cur);
        CUDA_TRY(cudaMemcpyAsync(r->d_cmove, cur.data(), (size_t)C * sizeof(uint32_t), cudaMemcpyHostToDevice,
                                 r->stream));
    }
    r->h_ice.swap(flags);
    return refresh_cells(r);
}

// ------------------------------------------------------------ MoveStats
// spherdist / spherdistDeg and cartdist (utils/geomutils.cpp:311-386), in
// the same operation order, for the distance from each cell to each of its
// neighbours (MoveStats::finalize adds them up, actions/MoveStats.cpp:196-203)
static double ms_spherdist(double dLon1, double dLat1, double dLon2, double dLat2, double dR) {
    const double dX1 = std::cos(dLon1) * std::cos(dLat1);
    const double dY1 = std::sin(dLon1) * std::cos(dLat1);
    const double dZ1 = std::sin(dLat1);
    const double dX2 = std::cos(dLon2) * std::cos(dLat2);
    const double dY2 = std::sin(dLon2) * std::cos(dLat2);
    const double dZ2 = std::sin(dLat2);
    double dProd = dX1 * dX2 + dY1 * dY2 + dZ1 * dZ2;
    if (dProd > 1) {
        dProd = 1;
    } else if (dProd < -1) {
        dProd = -1;
    }
    return dR * std::acos(dProd);
}

static double ms_distance(const double *lon, const double *lat, double R, bool cart, int a, int b) {
    if (cart) {
        const double dX = lon[b] - lon[a], dY = lat[b] - lat[a];
        return 1.0 * std::sqrt(dX * dX + dY * dY);
    }
    return ms_spherdist(lon[a] * kQPi / 180, lat[a] * kQPi / 180, lon[b] * kQPi / 180, lat[b] * kQPi / 180, R);
}

double qhg_host_move_distance(const double *lon, const double *lat, double radius, bool cartesian, int a, int b) {
    return ms_distance(lon, lat, radius, cartesian, a, b);
}

static void ms_free(qhg_run *r) {
    cudaFree(r->d_ms_hops); cudaFree(r->d_ms_chops); cudaFree(r->d_ms_dist); cudaFree(r->d_ms_time);
    cudaFree(r->d_ms_D); cudaFree(r->d_ms_cdist); cudaFree(r->d_ms_ckey);
    r->d_ms_hops = r->d_ms_chops = nullptr;
    r->d_ms_dist = r->d_ms_time = r->d_ms_D = nullptr;
    r->d_ms_cdist = r->d_ms_ckey = nullptr;
    r->ms_mode = -1;
}

// MoveStats::preLoop / initializeOccupied (actions/MoveStats.cpp:96-175):
// hops, distance and time -1, the cells of the current table 0; no candidates
static int ms_reset(qhg_run *r) {
    const int C = r->C;
    std::vector<int32_t> hops((size_t)C, -1), chops((size_t)C, INT32_MAX);
    std::vector<double> dt((size_t)C, -1.0);
    std::vector<unsigned long long> cdist((size_t)C, 0x7ff0000000000000ull);
    std::vector<unsigned long long> ckey((size_t)C, r->ms_mode == 0 ? ~0ull : 0ull);
    std::vector<double> dist(dt);
    if (r->agents_ok) {
        CUDA_TRY(cudaStreamSynchronize(r->stream));
        const uint32_t nne = r->h_rs->n_nonempty;
        std::vector<uint32_t> ne(nne);
        if (nne > 0) CUDA_TRY(cudaMemcpy(ne.data(), r->d_ne[r->cur], nne * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        for (uint32_t c : ne) {
            hops[c] = 0;
            dist[c] = 0.0;
            dt[c] = 0.0;
        }
    }
    cudaStream_t st = r->stream;
    CUDA_TRY(cudaMemcpyAsync(r->d_ms_hops, hops.data(), (size_t)C * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(r->d_ms_dist, dist.data(), (size_t)C * sizeof(double), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(r->d_ms_time, dt.data(), (size_t)C * sizeof(double), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(r->d_ms_chops, chops.data(), (size_t)C * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(r->d_ms_cdist, cdist.data(), (size_t)C * 8, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(r->d_ms_ckey, ckey.data(), (size_t)C * 8, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return QHG_OK;
}

extern "C" int qhg_gpu_move_stats_enable(qhg_run *r, int32_t mode, const double *lon, const double *lat,
                                         double radius, int32_t cartesian) {
    if (r == nullptr || lon == nullptr || lat == nullptr) return fail(QHG_ERR_ARG, "null argument");
    if (mode < QHG_MOVESTATS_FIRST || mode > QHG_MOVESTATS_LAST) return fail(QHG_ERR_ARG, "bad MoveStats mode");
    if (!r->grid_ok) return fail(QHG_ERR_STATE, "upload the grid first");
    CUDA_TRY(cudaSetDevice(r->desc.device));
    {
        const int hg = host_grid(r);   // the grid's host copies (fetched once)
        if (hg != QHG_OK) return hg;
    }
    int rc = pull_state(r);
    if (rc != QHG_OK) return rc;
    const int C = r->C;
    std::vector<double> D((size_t)C * 6, 0.0);
    for (int c = 0; c < C; c++) {
        for (int k = 0; k < (int)r->h_nnbr[c]; k++) {
            const int d = r->h_nbr[(size_t)c * 6 + k];
            if (d >= 0) D[(size_t)c * 6 + k] = ms_distance(lon, lat, radius, cartesian != 0, c, d);
        }
    }
    drop_graphs(r);   // the step graph gains the MoveStats kernels
    if (r->d_ms_hops == nullptr) {
        CUDA_TRY(cudaMalloc(&r->d_ms_hops, (size_t)C * sizeof(int32_t)));
        CUDA_TRY(cudaMalloc(&r->d_ms_chops, (size_t)C * sizeof(int32_t)));
        CUDA_TRY(cudaMalloc(&r->d_ms_dist, (size_t)C * sizeof(double)));
        CUDA_TRY(cudaMalloc(&r->d_ms_time, (size_t)C * sizeof(double)));
        CUDA_TRY(cudaMalloc(&r->d_ms_D, (size_t)C * 6 * sizeof(double)));
        CUDA_TRY(cudaMalloc(&r->d_ms_cdist, (size_t)C * 8));
        CUDA_TRY(cudaMalloc(&r->d_ms_ckey, (size_t)C * 8));
    }
    CUDA_TRY(cudaMemcpyAsync(r->d_ms_D, D.data(), D.size() * sizeof(double), cudaMemcpyHostToDevice, r->stream));
    r->ms_mode = mode;
    return ms_reset(r);
}

extern "C" int qhg_gpu_set_move_stats(qhg_run *r, const int32_t *hops, const double *dist, const double *time) {
    if (r == nullptr || hops == nullptr || dist == nullptr || time == nullptr) return fail(QHG_ERR_ARG, "null argument");
    if (r->ms_mode < 0) return fail(QHG_ERR_STATE, "MoveStats is not enabled");
    CUDA_TRY(cudaSetDevice(r->desc.device));
    int rc = pull_state(r);
    if (rc != QHG_OK) return rc;
    const size_t C = (size_t)r->C;
    CUDA_TRY(cudaMemcpyAsync(r->d_ms_hops, hops, C * sizeof(int32_t), cudaMemcpyHostToDevice, r->stream));
    CUDA_TRY(cudaMemcpyAsync(r->d_ms_dist, dist, C * sizeof(double), cudaMemcpyHostToDevice, r->stream));
    CUDA_TRY(cudaMemcpyAsync(r->d_ms_time, time, C * sizeof(double), cudaMemcpyHostToDevice, r->stream));
    CUDA_TRY(cudaStreamSynchronize(r->stream));
    return QHG_OK;
}

extern "C" int qhg_gpu_move_stats(qhg_run *r, int32_t *hops, double *dist, double *time) {
    if (r == nullptr || hops == nullptr || dist == nullptr || time == nullptr) return fail(QHG_ERR_ARG, "null argument");
    if (r->ms_mode < 0) return fail(QHG_ERR_STATE, "MoveStats is not enabled");
    CUDA_TRY(cudaSetDevice(r->desc.device));
    int rc = pull_state(r);
    if (rc != QHG_OK) return rc;
    const size_t C = (size_t)r->C;
    CUDA_TRY(cudaMemcpy(hops, r->d_ms_hops, C * sizeof(int32_t), cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(dist, r->d_ms_dist, C * sizeof(double), cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(time, r->d_ms_time, C * sizeof(double), cudaMemcpyDeviceToHost));
    return QHG_OK;
}

extern "C" int qhg_gpu_num_agents(qhg_run *r, int64_t *n) {
    if (r == nullptr || n == nullptr) return fail(QHG_ERR_ARG, "null argument");
    int rc = qhg_gpu_sync(r);
    if (rc != QHG_OK) return rc;
    *n = r->agents_ok ? (int64_t)r->h_rs->n_agents : 0;
    return QHG_OK;
}

extern "C" int qhg_gpu_current_step(qhg_run *r, int32_t *step) {
    if (r == nullptr || step == nullptr) return fail(QHG_ERR_ARG, "null argument");
    int rc = qhg_gpu_sync(r);
    if (rc != QHG_OK) return rc;
    *step = r->h_rs->step;
    return QHG_OK;
}

extern "C" int qhg_gpu_download(qhg_run *r, qhg_agents_soa *o, int64_t cap, int64_t *n) {
    if (r == nullptr || o == nullptr || n == nullptr) return fail(QHG_ERR_ARG, "null argument");
    if (!r->agents_ok) return fail(QHG_ERR_STATE, "no agents uploaded");
    int rc = qhg_gpu_sync(r);
    if (rc != QHG_OK) return rc;
    const int64_t N = r->h_rs->n_agents;
    *n = N;
    if (cap < N) return fail(QHG_ERR_ARG, "output arrays too small");
    const int cur = r->cur;
    const uint32_t nne = r->h_rs->n_nonempty;
    if (N > 0) {
        // per-row columns built on the device, in the step's scratch arrays
        // (the outcome words hold the cells, the father rows gender and state;
        // the next step's action kernel writes both before reading them); the
        // table's ages, where derived (t - birth of the step that made the
        // table, GetOld's fp32 arithmetic, actions/GetOld.cpp:44), into its
        // own age column
        int32_t *d_cell = reinterpret_cast<int32_t *>(r->d_outc);
        uint8_t *d_gender = reinterpret_cast<uint8_t *>(r->d_father);
        uint8_t *d_state = d_gender + r->cap;
        const int le = qhg_launch_download_cols(r->d_ne[cur], r->d_nes[cur], nne, (uint32_t)N, r->d_meta[cur],
                                                r->d_birth[cur], (float)(r->h_rs->step - 1),
                                                r->h_rs->age_derived ? 1 : 0, d_cell, d_gender, d_state,
                                                r->d_age[cur], r->stream);
        if (le != 0) return fail(QHG_ERR_CUDA, std::string("launch: ") + cudaGetErrorString((cudaError_t)le));
        cudaStream_t st = r->stream;
        CUDA_TRY(cudaMemcpyAsync(o->id, r->d_id[cur], N * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaMemcpyAsync(o->cell, d_cell, N * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaMemcpyAsync(o->birth, r->d_birth[cur], N * sizeof(float), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaMemcpyAsync(o->age, r->d_age[cur], N * sizeof(float), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaMemcpyAsync(o->last_birth, r->d_lastb[cur], N * sizeof(float), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaMemcpyAsync(o->gender, d_gender, N, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaMemcpyAsync(o->state, d_state, N, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
    }
    if (r->P.genome_words > 0 && o->genome != nullptr && N > 0) {
        const size_t gw = (size_t)r->P.genome_words;
        uint64_t *tmp = nullptr;
        CUDA_TRY(cudaMalloc(&tmp, (size_t)N * gw * sizeof(uint64_t)));
        int le = qhg_launch_gather_genomes(r->d_gslot[cur], r->d_genome, (uint32_t)N, r->P.genome_words,
                                           r->gcap, tmp, r->stream);
        cudaError_t e = le == 0 ? cudaStreamSynchronize(r->stream) : (cudaError_t)le;
        if (e == cudaSuccess) e = cudaMemcpy(o->genome, tmp, (size_t)N * gw * sizeof(uint64_t), cudaMemcpyDeviceToHost);
        cudaFree(tmp);
        if (e != cudaSuccess) return fail(QHG_ERR_CUDA, std::string("genome gather: ") + cudaGetErrorString(e));
    }
    return QHG_OK;
}

extern "C" int qhg_gpu_counts(qhg_run *r, uint32_t *counts) {
    if (r == nullptr || counts == nullptr) return fail(QHG_ERR_ARG, "null argument");
    if (!r->agents_ok) return fail(QHG_ERR_STATE, "no agents uploaded");
    int rc = qhg_gpu_sync(r);
    if (rc != QHG_OK) return rc;
    const uint32_t nne = r->h_rs->n_nonempty;
    std::vector<uint32_t> ne(nne), nes((size_t)nne + 1);
    if (nne > 0) CUDA_TRY(cudaMemcpy(ne.data(), r->d_ne[r->cur], nne * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(nes.data(), r->d_nes[r->cur], (nne + 1) * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    for (int c = 0; c < r->C; c++) counts[c] = 0u;
    for (uint32_t k = 0; k < nne; k++) counts[ne[k]] = nes[(size_t)k + 1] - nes[k];
    return QHG_OK;
}

extern "C" int qhg_gpu_occupancy(qhg_run *r, int32_t *first_step) {
    if (r == nullptr || first_step == nullptr) return fail(QHG_ERR_ARG, "null argument");
    if (r->d_occ == nullptr) return fail(QHG_ERR_STATE, "run was created without QHG_FLAG_TRACK_OCCUPANCY");
    int rc = qhg_gpu_sync(r);
    if (rc != QHG_OK) return rc;
    CUDA_TRY(cudaMemcpy(first_step, r->d_occ, (size_t)r->C * sizeof(int32_t), cudaMemcpyDeviceToHost));
    return QHG_OK;
}

extern "C" int qhg_gpu_set_occupancy(qhg_run *r, const int32_t *first_step) {
    if (r == nullptr || first_step == nullptr) return fail(QHG_ERR_ARG, "null argument");
    if (r->d_occ == nullptr) return fail(QHG_ERR_STATE, "run was created without QHG_FLAG_TRACK_OCCUPANCY");
    int rc = qhg_gpu_sync(r);
    if (rc != QHG_OK) return rc;
    CUDA_TRY(cudaMemcpy(r->d_occ, first_step, (size_t)r->C * sizeof(int32_t), cudaMemcpyHostToDevice));
    return QHG_OK;
}

extern "C" int qhg_gpu_stats(qhg_run *r, int32_t nsteps, qhg_step_stats *out) {
    if (r == nullptr || out == nullptr || nsteps < 0 || nsteps > kStatsRing) return fail(QHG_ERR_ARG, "bad stats arguments");
    int rc = qhg_gpu_sync(r);
    if (rc != QHG_OK) return rc;
    const int32_t st = r->h_rs->step;
    for (int32_t k = 0; k < nsteps; k++) {
        const uint32_t s = (uint32_t)(st - nsteps + k);
        const unsigned long long *v = r->h_rs->stats[s % kStatsRing];
        out[k].live = v[0]; out[k].births = v[1]; out[k].deaths = v[2]; out[k].moves = v[3];
    }
    return QHG_OK;
}

extern "C" int qhg_gpu_stats_async(qhg_run *r, qhg_step_stats *out) {
    if (r == nullptr || out == nullptr) return fail(QHG_ERR_ARG, "null argument");
    if (!r->agents_ok || r->launched == 0) return fail(QHG_ERR_STATE, "no step launched since the last sync");
    CUDA_TRY(cudaSetDevice(r->desc.device));
    const uint32_t s = (uint32_t)(r->h_rs->step + r->launched - 1);
    const char *src = reinterpret_cast<const char *>(r->d_rs) + offsetof(RunState, stats) +
                      (size_t)(s % kStatsRing) * 4 * sizeof(unsigned long long);
    static_assert(sizeof(qhg_step_stats) == 4 * sizeof(unsigned long long), "stats layout");
    CUDA_TRY(cudaMemcpyAsync(out, src, sizeof(qhg_step_stats), cudaMemcpyDeviceToHost, r->stream));
    return QHG_OK;
}

extern "C" int qhg_gpu_birth_log(qhg_run *r, int64_t *baby, int64_t *mother, int64_t *father, int64_t cap,
                                 int64_t *n) {
    if (r == nullptr || n == nullptr) return fail(QHG_ERR_ARG, "null argument");
    if (!r->P.log_births) return fail(QHG_ERR_STATE, "run was created without QHG_FLAG_LOG_BIRTHS");
    int rc = qhg_gpu_sync(r);
    if (rc != QHG_OK) return rc;
    const uint64_t total = r->h_rs->birth_log_n;
    *n = (int64_t)total;
    if (total > r->blog_cap) return fail(QHG_ERR_CAPACITY, "birth log overflowed");
    if ((uint64_t)cap < total) return fail(QHG_ERR_ARG, "output arrays too small");
    std::vector<int64_t> tmp(total * 3);
    if (total > 0) {
        CUDA_TRY(cudaMemcpy(tmp.data(), r->d_blog, total * 3 * sizeof(int64_t), cudaMemcpyDeviceToHost));
    }
    for (uint64_t i = 0; i < total; i++) {
        baby[i] = tmp[i * 3]; mother[i] = tmp[i * 3 + 1]; father[i] = tmp[i * 3 + 2];
    }
    return QHG_OK;
}

extern "C" int qhg_gpu_next_id(qhg_run *r, int64_t *next_id) {
    if (r == nullptr || next_id == nullptr) return fail(QHG_ERR_ARG, "null argument");
    int rc = qhg_gpu_sync(r);
    if (rc != QHG_OK) return rc;
    *next_id = r->h_rs->next_id;
    return QHG_OK;
}

extern "C" int qhg_gpu_set_next_id(qhg_run *r, int64_t next_id) {
    if (r == nullptr) return fail(QHG_ERR_ARG, "null run");
    if (!r->agents_ok) return fail(QHG_ERR_STATE, "upload the agents first");
    int rc = qhg_gpu_sync(r);
    if (rc != QHG_OK) return rc;
    if (next_id < r->upload_max_id + 1) return fail(QHG_ERR_ARG, "next ID not above every live agent's ID");
    CUDA_TRY(cudaMemcpyAsync(reinterpret_cast<char *>(r->d_rs) + offsetof(RunState, next_id), &next_id,
                             sizeof(int64_t), cudaMemcpyHostToDevice, r->stream));
    CUDA_TRY(cudaStreamSynchronize(r->stream));
    r->h_rs->next_id = next_id;
    return QHG_OK;
}

extern "C" int qhg_gpu_test_stall_scan(qhg_run *r, int32_t tile) {
    if (r == nullptr) return fail(QHG_ERR_ARG, "null run");
    const int ntiles = (r->C + kScanTile - 1) / kScanTile;
    if (tile < 0 || tile >= ntiles - 1) return fail(QHG_ERR_ARG, "the tile must have a successor");
    CUDA_TRY(cudaSetDevice(r->desc.device));
    const uint32_t v = (uint32_t)tile + 1u;
    CUDA_TRY(cudaMemcpyAsync(reinterpret_cast<char *>(r->d_rs) + offsetof(RunState, stall_tile), &v,
                             sizeof(uint32_t), cudaMemcpyHostToDevice, r->stream));
    CUDA_TRY(cudaStreamSynchronize(r->stream));
    return QHG_OK;
}

extern "C" int qhg_gpu_stream(qhg_run *r, void **stream) {
    if (r == nullptr || stream == nullptr) return fail(QHG_ERR_ARG, "null argument");
    *stream = (void *)r->stream;
    return QHG_OK;
}

extern "C" int qhg_gpu_destroy(qhg_run *r) {
    if (r == nullptr) return QHG_OK;
    cudaSetDevice(r->desc.device);
    if (r->stream) cudaStreamSynchronize(r->stream);
    drop_graphs(r);
    free_agents(r);
    cudaFree(r->d_nbr); cudaFree(r->d_nnbr); cudaFree(r->d_rev); cudaFree(r->d_K); cudaFree(r->d_vthr[0]); cudaFree(r->d_vthr[1]);
    cudaFree(r->d_wthr); cudaFree(r->d_cmove); cudaFree(r->d_occ);
    cudaFree(r->d_clsc); cudaFree(r->d_sbase); cudaFree(r->d_bbase); cudaFree(r->d_bidb);
    cudaFree(r->d_obase); cudaFree(r->d_tflag); cudaFree(r->d_tagg); cudaFree(r->d_tincl);
    ms_free(r);
    cudaFree(r->d_rs);
    cudaFreeHost(r->h_rs);
    for (int i = 0; i < 5; i++) {
        if (r->ev[i]) cudaEventDestroy(r->ev[i]);
    }
    if (r->stream) cudaStreamDestroy(r->stream);
    delete r;
    return QHG_OK;
}
