/*
 * CPU restatement of QHG4's per-step agent hot path ("port" oracle).
 *
 * ORACLE / TEST INFRASTRUCTURE ONLY.  Used by tests/ as the checker of the
 * CUDA path, by __graft_entry__.smoke() and by bench.py's CPU-baseline and
 * reference legs.  Nothing in the product links or loads it.  It is pinned
 * against the reference's own action code (the Philox test build in
 * oracle/ref/, see tests/test_oracle_pinning.py and tests/golden/).
 *
 * One step = the reference's PopLooper::doStep (core/PopLooper.cpp:166-200):
 *   initializeStep  per-cell Verhulst rates (actions/LinearBirth.cpp:90-112,
 *                   actions/LinearDeath.cpp:92-122), WeightedMove weights
 *                   (actions/SingleEvaluator.cpp:174-241) and pairing
 *                   (actions/RandomPair.cpp:107-270, keyed by agent ID)
 *   doActions       the actions in execution order on every live agent
 *                   (core/SPopulation.cpp:554-577); an agent that dies skips
 *                   the rest (core/SPopulation.cpp:568, :934)
 *   finalizeStep    births (core/SPopulation.cpp:596-724, 880-918), moves
 *                   (core/SPopulation.cpp:1014-1092), per-cell counts
 *                   (core/SPopulation.cpp:509-536)
 * Draws: Philox4x32-10 keyed by (seed, step, agent ID, action window), see
 * philox4x32.h.  Births are numbered in (cell, mother ID) order.
 *
 * Agents are kept sorted by ID (survivors keep their order, newborns get
 * larger IDs and are appended), so every per-cell list built by a stable
 * pass over the agents is in ID order.
 *
 * Compile with -ffp-contract=off: the decision arithmetic must round like
 * the reference's.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <stdio.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "philox4x32.h"

enum {
    ACT_GETOLD = 0, ACT_FERTILITY = 1, ACT_RANDOMPAIR = 2, ACT_VERHULST = 3,
    ACT_VERHULSTVARK = 4, ACT_OLDAGEDEATH = 5, ACT_RANDOMMOVE = 6, ACT_WEIGHTEDMOVE = 7,
    ACT_ATANDEATH = 8
};
#define MAX_ACTIONS 16
#define CROSSOVER_POISSON1 (-100)
#define LS_DEAD 0u
#define LS_ALIVE 1u
#define LS_FERTILE 5u
#define TWO32 4294967296.0
/* Q_PI (utils/qhg_consts.h): std::numbers::pi, the double nearest pi */
#define QO_PI 3.141592653589793

/* Poisson(1) inverse-CDF thresholds floor(P(K<=k) * 2^32), exact */
static const uint32_t POISSON1_CDF32[16] = {
    1580030168u, 3160060337u, 3950075421u, 4213413783u, 4279248373u,
    4292415291u, 4294609777u, 4294923276u, 4294962463u, 4294966817u,
    4294967252u, 4294967292u, 4294967295u, 4294967295u, 4294967295u,
    4294967295u
};

typedef struct {
    /* configuration */
    uint64_t seed;
    int n_act;
    int act_type[MAX_ACTIONS];
    double act_p[MAX_ACTIONS][4];
    double act_scale[MAX_ACTIONS];   /* ATanDeath: m_dScale of preLoop */
    uint32_t act_window[MAX_ACTIONS];
    int has_pair;
    int genome_size, num_blocks, num_crossover;
    double mutation_rate;
    double *bino;       /* BinomialDist lookup table */
    int n_bino;
    /* grid */
    int C;
    int32_t *nbr;
    uint8_t *nnbr;
    double *K;
    double *W;          /* cumulated WeightedMove weights [C*7] */
    int w_given;        /* W was given (qo_set_move_weights), not derived from K */
    uint8_t *ice;       /* Geography::m_abIce per cell (NULL: no Geography, no ice) */
    /* agents, sorted by ID */
    int64_t n, cap;
    int64_t *id;
    int32_t *cell;
    float *birth, *age, *lastb;
    uint8_t *gender, *state;
    int32_t *gslot;     /* genome slot of each agent row */
    uint64_t *genome;   /* genome slab [gcap slots * 2 * num_blocks]; slots, not rows, hold genomes,
                         * as the reference's LayerArrBuf does, so rows move without their genomes */
    int64_t gcap, ghwm; /* slots allocated, slots ever used */
    int32_t *gfree;     /* free slots (of agents that died in earlier steps) */
    int64_t nfree;
    int64_t next_id;
    /* per cell */
    uint32_t *count;
    double *B, *D;
    /* step */
    int32_t step;
    uint64_t *stats;    /* 4 per step done */
    int64_t stats_cap;
    int64_t *blog;      /* birth log: baby, mother, father */
    int64_t blog_n, blog_cap;
    int log_births;
    /* MoveStats (actions/MoveStats.h): mode -1 none, 0 first, 1 min, 2 last;
     * cell coordinates (degrees, or plane x/y), the definitive per-cell hops,
     * distance and time, and the temporaries that persist between steps */
    int ms_mode;
    int ms_cart;
    double ms_R;
    double *ms_lon, *ms_lat;
    int32_t *ms_hops, *ms_thops;
    double *ms_dist, *ms_time, *ms_tdist, *ms_ttime;
    uint8_t *ms_changed;
} qo_run;

/* ---------------------------------------------------------------- draws */
static inline double u2d(uint32_t u) { return (1.0 * u) / TWO32; }

typedef struct { uint64_t seed; uint32_t step; int64_t id; uint32_t base; uint32_t k; } stream_t;

static inline uint32_t next_draw(stream_t *s) {
    return qhg_oracle_draw(s->seed, s->step, s->id, s->base, s->k++);
}

/* ------------------------------------------------- binomial lookup table */
/* Numerical Recipes' incomplete beta (gammln, betacf, betai), the algorithm
 * the reference uses in utils/bino_tools.cpp, restated. */
static double nr_gammaln(double xx) {
    static const double cof[6] = {76.18009172947146, -86.50532032941677, 24.01409824083091,
                                  -1.231739572450155, 0.1208650973866179e-2, -0.5395239384953e-5};
    double ser = 1.000000000190015;
    double x = xx;
    double y = xx + 1;
    double tmp = x + 5.5;
    tmp -= (x + 0.5) * log(tmp);
    for (int k = 0; k <= 5; k++) {
        ser += cof[k] / y;
        y++;
    }
    return -tmp + log(2.5066282746310005 * ser / x);
}

static double nr_betacf(double a, double b, double x) {
    const double FMIN = 1.0e-30f;
    double qab = a + b, qap = a + 1.0, qam = a - 1.0;
    double c = 1.0;
    double d = 1.0 - qab * x / qap;
    if (fabs(d) < FMIN) d = FMIN;
    d = 1.0 / d;
    double h = d;
    int m;
    for (m = 1; m <= 100; m++) {
        int m2 = 2 * m;
        double aa = m * (b - m) * x / ((qam + m2) * (a + m2));
        d = 1.0 + aa * d;
        if (fabs(d) < FMIN) d = FMIN;
        c = 1.0 + aa / c;
        if (fabs(c) < FMIN) c = FMIN;
        d = 1.0 / d;
        h *= d * c;
        aa = -(a + m) * (qab + m) * x / ((a + m2) * (qap + m2));
        d = 1.0 + aa * d;
        if (fabs(d) < FMIN) d = FMIN;
        c = 1.0 + aa / c;
        if (fabs(c) < FMIN) c = FMIN;
        d = 1.0 / d;
        double del = d * c;
        h *= del;
        if (fabs(del - 1.0) < 3.0e-7) break;
    }
    if (m > 100) h = -1;
    return h;
}

static double nr_beta(double a, double b, double x) {
    double bt;
    if ((x < 0.0) || (x > 1.0)) return -1;
    if ((x == 0.0) || (x == 1.0)) {
        bt = 0.0;
    } else {
        bt = exp(nr_gammaln(a + b) - nr_gammaln(a) - nr_gammaln(b) + a * log(x) + b * log(1.0 - x));
    }
    if (x < (a + 1.0) / (a + b + 2.0)) {
        return bt * nr_betacf(a, b, x) / a;
    }
    return 1.0 - bt * nr_betacf(b, a, 1.0 - x) / b;
}

/* BinomialDist::buildTable (utils/BinomialDist.cpp:61-89) */
static int build_bino(qo_run *r, double p, int n, double eps) {
    int cap = 64, cnt = 0;
    double *v = (double *)malloc(cap * sizeof(double));
    int k = 1;
    double d2 = nr_beta(k, n - k + 1, p);
    while ((d2 > eps) && (k < n)) {
        if (cnt == cap) { cap *= 2; v = (double *)realloc(v, cap * sizeof(double)); }
        v[cnt++] = d2;
        k++;
        d2 = nr_beta(k, n - k + 1, p);
    }
    if (cnt == cap) { cap *= 2; v = (double *)realloc(v, cap * sizeof(double)); }
    v[cnt++] = d2;
    for (int i = 0; i < cnt; i++) v[i] = 1 - v[i];
    r->bino = v;
    r->n_bino = cnt;
    return 0;
}

/* BinomialDist::getN (utils/BinomialDist.cpp:92-104) */
static int bino_getN(const qo_run *r, double dP) {
    int i = 0;
    while ((i < r->n_bino) && (dP > r->bino[i])) i++;
    return i;
}

/* ------------------------------------------------------------ genetics */
/* BitGeneUtils::makeMultiMask (genes/BitGeneUtils.cpp:90-109), including
 * its behaviour for breaks that are not in ascending order */
static uint64_t multi_mask(const uint32_t *br, int nb) {
    uint32_t k = 1 - (uint32_t)(nb % 2);
    uint64_t out = 0;
    int i = nb - 1;
    for (uint32_t j = 0; j < 64; j++) {
        if ((i >= 0) && (j == 64u - br[i])) {
            i--;
            k = 1 - k;
        }
        out = (out << 1) + k;
    }
    return out;
}

/* BitGeneUtils::crossOver (genes/BitGeneUtils.cpp:116-188) for 1-bit loci:
 * breaks drawn with wrandi(0, nblocks*64) in draw order, grouped per block */
static void cross_over(uint64_t *dst, const uint64_t *g, int nblk, int nbreaks, stream_t *s) {
    uint32_t blk[64], bit[64];
    if (nbreaks > 64) nbreaks = 64;
    uint32_t nbits = (uint32_t)nblk * 64u;
    for (int i = 0; i < nbreaks; i++) {
        uint32_t u = next_draw(s);
        uint32_t pos = (uint32_t)((1.0 * nbits * u) / (1.0 * TWO32));
        blk[i] = pos / 64u;
        bit[i] = pos % 64u;
    }
    int before = 0;
    for (int b = 0; b < nblk; b++) {
        uint32_t br[64];
        int nb = 0;
        for (int i = 0; i < nbreaks; i++) {
            if (blk[i] == (uint32_t)b) br[nb++] = bit[i];
        }
        int cur = before % 2;
        uint64_t m = (nb > 0) ? multi_mask(br, nb) : ~0ULL;
        uint64_t a = g[cur * nblk + b], o = g[(1 - cur) * nblk + b];
        dst[b] = (m & a) | (~m & o);
        dst[nblk + b] = (m & o) | (~m & a);
        before += nb;
    }
}

static int poisson1(uint32_t u) {
    int k = 0;
    while (k < 16 && u >= POISSON1_CDF32[k]) k++;
    return k;
}

/* Genetics::makeOffspring (actions/Genetics.cpp:285-337); draws continue the
 * birth stream after the gender draw */
static void make_genome(const qo_run *r, uint64_t *baby, const uint64_t *gm, const uint64_t *gf, stream_t *s) {
    int nblk = r->num_blocks;
    uint64_t t1[2 * 64 * 64], t2[2 * 64 * 64];
    int i1 = (int)(2 * 1.0 * u2d(next_draw(s)));
    int i2 = (int)(2 * 1.0 * u2d(next_draw(s)));
    const uint64_t *s1 = gm, *s2 = gf;
    if (r->num_crossover == CROSSOVER_POISSON1) {
        int nm = poisson1(next_draw(s));
        int nf = poisson1(next_draw(s));
        cross_over(t1, gm, nblk, nm, s);
        cross_over(t2, gf, nblk, nf, s);
        s1 = t1; s2 = t2;
    } else if (r->num_crossover > 0) {
        cross_over(t1, gm, nblk, r->num_crossover, s);
        cross_over(t2, gf, nblk, r->num_crossover, s);
        s1 = t1; s2 = t2;
    }
    memcpy(baby, s1 + i1 * nblk, nblk * sizeof(uint64_t));
    memcpy(baby + nblk, s2 + i2 * nblk, nblk * sizeof(uint64_t));
    if (r->mutation_rate > 0) {
        int nmut = bino_getN(r, u2d(next_draw(s)));
        uint32_t nbits = 2u * (uint32_t)r->genome_size;
        for (int i = 0; i < nmut; i++) {
            uint32_t pos = (uint32_t)((1.0 * nbits * next_draw(s)) / (1.0 * TWO32));
            baby[pos / 64u] ^= 1ULL << (pos % 64u);
        }
    }
}

/* WeightedMove's weights from K: a SingleEvaluator with direct values,
 * cumulated over the neighbours (actions/SingleEvaluator.cpp:174-241); an
 * ice cell of the Geography weighs 0 (:183-202) */
static void weights_from_K(qo_run *r) {
    const int C = r->C;
    for (int c = 0; c < C; c++) {
        double dV = r->K[c];
        r->W[(size_t)c * 7] = (r->ice != NULL && r->ice[c]) ? 0 : ((dV > 0) ? dV : 0);
    }
    for (int c = 0; c < C; c++) {
        double dW = r->W[(size_t)c * 7];
        for (int i = 0; i < 6; i++) {
            double dCW = 0;
            int ni = r->nbr[(size_t)c * 6 + i];
            if (ni >= 0) dCW = r->W[(size_t)ni * 7];
            dCW = (dCW > 0) ? dCW : 0;
            dW = dW + dCW;
            r->W[(size_t)c * 7 + i + 1] = dW;
        }
    }
}

/* ------------------------------------------------------------ MoveStats */
/* spherdist / spherdistDeg and cartdist (utils/geomutils.cpp:311-386),
 * restated in the same operation order */
static double ms_spherdist(double dLon1, double dLat1, double dLon2, double dLat2, double dR) {
    double dX1 = cos(dLon1) * cos(dLat1);
    double dY1 = sin(dLon1) * cos(dLat1);
    double dZ1 = sin(dLat1);
    double dX2 = cos(dLon2) * cos(dLat2);
    double dY2 = sin(dLon2) * cos(dLat2);
    double dZ2 = sin(dLat2);
    double dProd = dX1 * dX2 + dY1 * dY2 + dZ1 * dZ2;
    if (dProd > 1) {
        dProd = 1;
    } else if (dProd < -1) {
        dProd = -1;
    }
    return dR * acos(dProd);
}

static double ms_distance(const qo_run *r, int a, int b) {
    if (r->ms_cart) {
        double dX = r->ms_lon[b] - r->ms_lon[a], dY = r->ms_lat[b] - r->ms_lat[a];
        return 1.0 * sqrt(dX * dX + dY * dY);
    }
    return ms_spherdist(r->ms_lon[a] * QO_PI / 180, r->ms_lat[a] * QO_PI / 180,
                        r->ms_lon[b] * QO_PI / 180, r->ms_lat[b] * QO_PI / 180, r->ms_R);
}

/* MoveStats::preLoop / initializeOccupied (actions/MoveStats.cpp:96-175):
 * everything -1, the cells holding agents 0 */
static void ms_init(qo_run *r) {
    for (int c = 0; c < r->C; c++) {
        r->ms_hops[c] = -1; r->ms_dist[c] = -1; r->ms_time[c] = -1;
        r->ms_thops[c] = -1; r->ms_tdist[c] = -1; r->ms_ttime[c] = -1;
    }
    for (int64_t i = 0; i < r->n; i++) {
        int c = r->cell[i];
        r->ms_hops[c] = 0; r->ms_dist[c] = 0; r->ms_time[c] = 0;
    }
}

/* ------------------------------------------------------------ create */
qo_run *qo_create(uint64_t seed, int n_act, const int32_t *types, const double *params,
                  int genome_size, int num_crossover, double mutation_rate,
                  int C, const int32_t *nbr, const uint8_t *nnbr, const double *K) {
    if (n_act < 0 || n_act > MAX_ACTIONS || C <= 0) return NULL;
    qo_run *r = (qo_run *)calloc(1, sizeof(qo_run));
    r->seed = seed;
    r->ms_mode = -1;
    r->n_act = n_act;
    uint32_t w = 0;
    for (int a = 0; a < n_act; a++) {
        r->act_type[a] = types[a];
        for (int k = 0; k < 4; k++) r->act_p[a][k] = params[a * 4 + k];
        r->act_window[a] = w;
        switch (types[a]) {
        case ACT_VERHULST: case ACT_VERHULSTVARK: case ACT_RANDOMMOVE: case ACT_WEIGHTEDMOVE: w += 2; break;
        case ACT_OLDAGEDEATH: w += 1; break;
        case ACT_ATANDEATH:
            /* ATanDeath::preLoop (actions/ATanDeath.cpp:41):
             * scale = (pi/2 - EPS) / atan(slope * range), EPS = 0.001
             * (actions/ATanDeath.h) */
            r->act_scale[a] = (QO_PI / 2 - 0.001) / atan(r->act_p[a][2] * r->act_p[a][1]);
            w += 1;
            break;
        case ACT_RANDOMPAIR: r->has_pair = 1; break;
        default: break;
        }
    }
    r->genome_size = genome_size;
    r->num_blocks = (genome_size > 0) ? (genome_size + 63) / 64 : 0;
    r->num_crossover = num_crossover;
    r->mutation_rate = mutation_rate;
    if (genome_size > 0) {
        if (r->num_blocks > 64) { free(r); return NULL; }
        build_bino(r, mutation_rate, 2 * genome_size, 1e-6);
    }
    r->C = C;
    r->nbr = (int32_t *)malloc((size_t)C * 6 * sizeof(int32_t));
    memcpy(r->nbr, nbr, (size_t)C * 6 * sizeof(int32_t));
    r->nnbr = (uint8_t *)malloc(C);
    memcpy(r->nnbr, nnbr, C);
    r->K = (double *)malloc(C * sizeof(double));
    memcpy(r->K, K, C * sizeof(double));
    r->W = (double *)calloc((size_t)C * 7, sizeof(double));
    weights_from_K(r);
    r->count = (uint32_t *)calloc(C, sizeof(uint32_t));
    r->B = (double *)calloc(C, sizeof(double));
    r->D = (double *)calloc(C, sizeof(double));
    r->log_births = 1;
    return r;
}

static void reserve_agents(qo_run *r, int64_t need) {
    if (need <= r->cap) return;
    int64_t cap = r->cap ? r->cap : 1024;
    while (cap < need) cap *= 2;
    r->id = (int64_t *)realloc(r->id, cap * sizeof(int64_t));
    r->cell = (int32_t *)realloc(r->cell, cap * sizeof(int32_t));
    r->birth = (float *)realloc(r->birth, cap * sizeof(float));
    r->age = (float *)realloc(r->age, cap * sizeof(float));
    r->lastb = (float *)realloc(r->lastb, cap * sizeof(float));
    r->gender = (uint8_t *)realloc(r->gender, cap);
    r->state = (uint8_t *)realloc(r->state, cap);
    if (r->num_blocks > 0) r->gslot = (int32_t *)realloc(r->gslot, cap * sizeof(int32_t));
    r->cap = cap;
}

/* room for `need` genome slots in the slab */
static void reserve_slots(qo_run *r, int64_t need) {
    if (need <= r->gcap) return;
    int64_t cap = r->gcap ? r->gcap : 1024;
    while (cap < need) cap *= 2;
    r->genome = (uint64_t *)realloc(r->genome, (size_t)cap * 2 * r->num_blocks * sizeof(uint64_t));
    r->gfree = (int32_t *)realloc(r->gfree, cap * sizeof(int32_t));
    r->gcap = cap;
}

static void recount(qo_run *r) {
    memset(r->count, 0, r->C * sizeof(uint32_t));
    for (int64_t i = 0; i < r->n; i++) r->count[r->cell[i]]++;
}

/* agents may come in any order; they are stored sorted by ID */
int qo_load(qo_run *r, int64_t N, const int64_t *id, const int32_t *cell, const float *birth,
            const float *age, const float *lastb, const uint8_t *gender, const uint8_t *state,
            const uint64_t *genome, int32_t first_step) {
    int64_t *ord = (int64_t *)malloc((N > 0 ? N : 1) * sizeof(int64_t));
    for (int64_t i = 0; i < N; i++) ord[i] = i;
    /* insertion into ID order via a simple merge sort on indices */
    int64_t *tmp = (int64_t *)malloc((N > 0 ? N : 1) * sizeof(int64_t));
    for (int64_t width = 1; width < N; width *= 2) {
        for (int64_t lo = 0; lo < N; lo += 2 * width) {
            int64_t mid = lo + width < N ? lo + width : N;
            int64_t hi = lo + 2 * width < N ? lo + 2 * width : N;
            int64_t a = lo, b = mid, k = lo;
            while (a < mid && b < hi) tmp[k++] = (id[ord[a]] <= id[ord[b]]) ? ord[a++] : ord[b++];
            while (a < mid) tmp[k++] = ord[a++];
            while (b < hi) tmp[k++] = ord[b++];
        }
        memcpy(ord, tmp, N * sizeof(int64_t));
    }
    free(tmp);
    reserve_agents(r, N);
    if (r->num_blocks > 0) reserve_slots(r, N);
    r->ghwm = 0;
    r->nfree = 0;
    r->n = 0;
    int64_t maxid = -1;
    for (int64_t j = 0; j < N; j++) {
        int64_t i = ord[j];
        if (state[i] == LS_DEAD) continue;
        if (cell[i] < 0 || cell[i] >= r->C) { free(ord); return -2; }
        int64_t k = r->n++;
        r->id[k] = id[i]; r->cell[k] = cell[i]; r->birth[k] = birth[i]; r->age[k] = age[i];
        r->lastb[k] = lastb[i]; r->gender[k] = gender[i]; r->state[k] = state[i];
        if (r->num_blocks > 0) {
            r->gslot[k] = (int32_t)k;
            memcpy(r->genome + (size_t)k * 2 * r->num_blocks, genome + (size_t)i * 2 * r->num_blocks,
                   2 * r->num_blocks * sizeof(uint64_t));
        }
        if (id[i] > maxid) maxid = id[i];
    }
    free(ord);
    r->ghwm = r->n;
    r->next_id = maxid + 1;
    r->step = first_step;
    recount(r);
    if (r->ms_mode >= 0) ms_init(r);
    return 0;
}

/* --------------------------------------------------------------- step */
typedef struct {
    int32_t mate;      /* index of the mate or -1 */
    int32_t move_to;   /* new cell or -1 */
    uint8_t dead;
    uint8_t birth;
} outcome_t;

/* RandomPair::findMates semantics (actions/RandomPair.cpp:146-270), members
 * ordered by agent ID and each pick keyed by the picking member's ID */
static void do_pairing(qo_run *r, outcome_t *out) {
    int C = r->C;
    int64_t n = r->n;
    uint32_t *fs = (uint32_t *)calloc((size_t)C + 1, sizeof(uint32_t));
    uint32_t *ms = (uint32_t *)calloc((size_t)C + 1, sizeof(uint32_t));
    for (int64_t i = 0; i < n; i++) {
        if (r->state[i] == LS_FERTILE) {
            if (r->gender[i] == 0) fs[r->cell[i] + 1]++;
            else if (r->gender[i] == 1) ms[r->cell[i] + 1]++;
        }
    }
    for (int c = 0; c < C; c++) { fs[c + 1] += fs[c]; ms[c + 1] += ms[c]; }
    int64_t *fl = (int64_t *)malloc((fs[C] + 1) * sizeof(int64_t));
    int64_t *ml = (int64_t *)malloc((ms[C] + 1) * sizeof(int64_t));
    uint32_t *fp = (uint32_t *)malloc((size_t)C * sizeof(uint32_t));
    uint32_t *mp = (uint32_t *)malloc((size_t)C * sizeof(uint32_t));
    memcpy(fp, fs, C * sizeof(uint32_t));
    memcpy(mp, ms, C * sizeof(uint32_t));
    for (int64_t i = 0; i < n; i++) {     /* stable: lists in ID order */
        if (r->state[i] == LS_FERTILE) {
            if (r->gender[i] == 0) fl[fp[r->cell[i]]++] = i;
            else if (r->gender[i] == 1) ml[mp[r->cell[i]]++] = i;
        }
    }
#pragma omp parallel for schedule(dynamic, 256)
    for (int c = 0; c < C; c++) {
        int nF = (int)(fs[c + 1] - fs[c]);
        int nM = (int)(ms[c + 1] - ms[c]);
        if (nF <= 0 || nM <= 0) continue;
        const int64_t *S, *L;
        int nS, nL;
        if (nF <= nM) { S = fl + fs[c]; nS = nF; L = ml + ms[c]; nL = nM; }
        else          { S = ml + ms[c]; nS = nM; L = fl + fs[c]; nL = nF; }
        uint8_t *taken = (uint8_t *)calloc(nL, 1);
        int nRem = nL;
        for (int j = 0; j < nS && nRem > 0; j++) {
            uint32_t u = qhg_oracle_draw(r->seed, (uint32_t)r->step, r->id[S[j]], QHG_STREAM_PAIR, 0);
            int choose = (int)(0 + ((nRem - 0) * (double)u) / TWO32);
            int seen = -1, iL = -1;
            while (seen < choose) {
                iL++;
                if (!taken[iL]) seen++;
            }
            taken[iL] = 1;
            out[S[j]].mate = (int32_t)L[iL];
            out[L[iL]].mate = (int32_t)S[j];
            nRem--;
        }
        free(taken);
    }
    free(fs); free(ms); free(fl); free(ml); free(fp); free(mp);
}

static void ensure_stats(qo_run *r, int64_t nsteps_more) {
    int64_t need = (int64_t)(r->stats_cap / 4) + nsteps_more;
    (void)need;
}

int qo_step(qo_run *r, int nsteps, uint64_t *stats_out) {
    for (int st = 0; st < nsteps; st++) {
        const float fT = (float)r->step;
        const int C = r->C;
        const int64_t n = r->n;
        /* ---- initializeStep: rates */
        for (int a = 0; a < r->n_act; a++) {
            int t = r->act_type[a];
            if (t != ACT_VERHULST && t != ACT_VERHULSTVARK) continue;
            double b0 = r->act_p[a][0], d0 = r->act_p[a][1], th = r->act_p[a][2], Kc = r->act_p[a][3];
            for (int c = 0; c < C; c++) {
                double nc = (double)r->count[c];
                if (t == ACT_VERHULST) {
                    r->B[c] = b0 + (th - b0) * (nc / Kc);
                    r->D[c] = d0 + (th - d0) * (nc / Kc);
                } else if (r->K[c] <= 0) {
                    r->B[c] = 0;
                    r->D[c] = 1;
                } else {
                    r->B[c] = b0 + (th - b0) * (nc / r->K[c]);
                    r->D[c] = d0 + (th - d0) * (nc / r->K[c]);
                }
            }
        }
        outcome_t *out = (outcome_t *)malloc((n > 0 ? n : 1) * sizeof(outcome_t));
        for (int64_t i = 0; i < n; i++) { out[i].mate = -1; out[i].move_to = -1; out[i].dead = 0; out[i].birth = 0; }
        if (r->has_pair) do_pairing(r, out);

        /* ---- doActions */
        uint64_t nMoves = 0, nDeaths = 0;
#pragma omp parallel for reduction(+:nMoves,nDeaths) schedule(static)
        for (int64_t i = 0; i < n; i++) {
            uint8_t st8 = r->state[i];
            float age = r->age[i];
            const int c = r->cell[i];
            int alive = st8 > LS_DEAD;
            for (int a = 0; a < r->n_act && alive; a++) {
                const double *p = r->act_p[a];
                stream_t s = { r->seed, (uint32_t)r->step, r->id[i], QHG_STREAM_ACTIONS, r->act_window[a] };
                switch (r->act_type[a]) {
                case ACT_GETOLD:      /* actions/GetOld.cpp:37-48 */
                    age = fT - r->birth[i];
                    break;
                case ACT_FERTILITY: { /* actions/Fertility.cpp:49-73 */
                    float fmin = (float)p[0], fmax = (float)p[1], fib = (float)p[2];
                    if (r->gender[i] == 0) {
                        st8 = ((age > fmin) && (age < fmax) && ((fT - r->lastb[i]) > fib)) ? LS_FERTILE : LS_ALIVE;
                    } else {
                        st8 = (age > fmin) ? LS_FERTILE : LS_ALIVE;
                    }
                    break;
                }
                case ACT_VERHULST:
                case ACT_VERHULSTVARK: {
                    /* LinearBirth::execute (actions/LinearBirth.cpp:122-166) */
                    double Bc = r->B[c];
                    if (Bc > 0) {
                        if ((r->gender[i] == 0) && (out[i].mate >= 0)) {
                            if (u2d(next_draw(&s)) < Bc) out[i].birth = 1;
                        }
                    } else if (Bc < 0) {
                        if (u2d(next_draw(&s)) < -Bc) { alive = 0; }
                    }
                    /* LinearDeath::execute (actions/LinearDeath.cpp:131-150) */
                    if (alive) {
                        if (u2d(next_draw(&s)) < r->D[c]) alive = 0;
                    }
                    if (!alive) nDeaths++;
                    break;
                }
                case ACT_OLDAGEDEATH: { /* actions/OldAgeDeath.cpp:48-67 */
                    double M = p[0], U = p[1];
                    age = fT - r->birth[i];
                    double lo = 1 - U * M, hi = 1 + U * M;
                    double dR = lo + ((hi - lo) * next_draw(&s)) / TWO32;
                    if (age > M + dR) { alive = 0; nDeaths++; }
                    break;
                }
                case ACT_ATANDEATH: { /* actions/ATanDeath.cpp:57-77 */
                    double M = p[0], slope = p[2];
                    age = fT - r->birth[i];
                    double dProb = 0.5 + r->act_scale[a] * atan(slope * (age - M)) / QO_PI;
                    if (u2d(next_draw(&s)) < dProb) { alive = 0; nDeaths++; }
                    break;
                }
                case ACT_RANDOMMOVE: { /* actions/RandomMove.cpp:65-100 */
                    if (u2d(next_draw(&s)) < p[0]) {
                        int nn = r->nnbr[c];
                        int dir = (int)(u2d(next_draw(&s)) * (nn + 1));
                        if (dir > 0) {
                            int to = r->nbr[(size_t)c * 6 + dir - 1];
                            if (to >= 0) { out[i].move_to = to; nMoves++; }
                        }
                    }
                    break;
                }
                case ACT_WEIGHTEDMOVE: { /* actions/WeightedMove.cpp:45-106 */
                    if (u2d(next_draw(&s)) < p[0]) {
                        int nn = r->nnbr[c];
                        const double *Wc = r->W + (size_t)c * 7;
                        int dir = -1;
                        if (Wc[0] == Wc[nn]) {
                            uint32_t rr = (uint32_t)(nn + 1);
                            dir = (int)(uint32_t)((1.0 * rr * next_draw(&s)) / (1.0 * TWO32));
                        } else {
                            double dR2 = u2d(next_draw(&s)) * Wc[nn];
                            for (int k = 0; k < nn + 1; k++) {
                                if (dR2 < Wc[k]) { dir = k; break; }
                            }
                        }
                        if (dir > 0) {
                            int to = r->nbr[(size_t)c * 6 + dir - 1];
                            /* a move into an ice cell is not registered (actions/WeightedMove.cpp:91) */
                            if (to >= 0 && (r->ice == NULL || !r->ice[to])) { out[i].move_to = to; nMoves++; }
                        }
                    }
                    break;
                }
                default:
                    break;
                }
            }
            r->age[i] = age;
            r->state[i] = alive ? st8 : LS_DEAD;
            out[i].dead = !alive;
        }

        /* ---- MoveStats::finalize (actions/MoveStats.cpp:183-256) as one
         * thread runs it, moves in agent-ID order; every registered move
         * counts, also that of an agent a later action killed */
        if (r->ms_mode >= 0) {
            const int mode = r->ms_mode;
            memset(r->ms_changed, 0, (size_t)C);
            for (int64_t i = 0; i < n; i++) {
                if (out[i].move_to < 0) continue;
                const int from = r->cell[i], to = out[i].move_to;
                int32_t iNewHops = r->ms_hops[from] + 1;
                double dNewDist = r->ms_dist[from] + ms_distance(r, from, to);
                double dNewTime = fT;
                if ((r->ms_thops[to] < 0) || (mode == 2)) {
                    r->ms_thops[to] = iNewHops;
                    r->ms_tdist[to] = dNewDist;
                    r->ms_ttime[to] = dNewTime;
                    r->ms_changed[to] = 1;
                } else if (mode == 1) {
                    if (iNewHops < r->ms_thops[to]) r->ms_thops[to] = iNewHops;
                    if (dNewDist < r->ms_tdist[to]) r->ms_tdist[to] = dNewDist;
                    r->ms_ttime[to] = dNewTime;
                    r->ms_changed[to] = 1;
                }
            }
            for (int c = 0; c < C; c++) {
                if (!r->ms_changed[c]) continue;
                if ((r->ms_hops[c] < 0) || (mode == 2)) {
                    r->ms_hops[c] = r->ms_thops[c];
                    r->ms_dist[c] = r->ms_tdist[c];
                    r->ms_time[c] = r->ms_ttime[c];
                } else if (mode == 1) {
                    if (r->ms_thops[c] < r->ms_hops[c]) r->ms_hops[c] = r->ms_thops[c];
                    if (r->ms_tdist[c] < r->ms_dist[c]) r->ms_dist[c] = r->ms_tdist[c];
                    if (r->ms_ttime[c] < r->ms_time[c]) r->ms_time[c] = r->ms_ttime[c];
                }
            }
        }

        /* ---- finalizeStep: births in (cell, mother ID) order */
        uint32_t *bs = (uint32_t *)calloc((size_t)C + 1, sizeof(uint32_t));
        int64_t nb = 0;
        for (int64_t i = 0; i < n; i++) if (out[i].birth) { bs[r->cell[i] + 1]++; nb++; }
        for (int c = 0; c < C; c++) bs[c + 1] += bs[c];
        int64_t *mom = (int64_t *)malloc((nb > 0 ? nb : 1) * sizeof(int64_t));
        for (int64_t i = 0; i < n; i++) if (out[i].birth) mom[bs[r->cell[i]]++] = i;
        free(bs);
        int64_t nsurv = 0;
        for (int64_t i = 0; i < n; i++) if (!out[i].dead) nsurv++;
        int64_t nnew = nsurv + nb;
        /* new arrays: survivors in ID order, then newborns */
        int64_t *id2 = (int64_t *)malloc((nnew > 0 ? nnew : 1) * sizeof(int64_t));
        int32_t *cell2 = (int32_t *)malloc((nnew > 0 ? nnew : 1) * sizeof(int32_t));
        float *birth2 = (float *)malloc((nnew > 0 ? nnew : 1) * sizeof(float));
        float *age2 = (float *)malloc((nnew > 0 ? nnew : 1) * sizeof(float));
        float *lastb2 = (float *)malloc((nnew > 0 ? nnew : 1) * sizeof(float));
        uint8_t *gender2 = (uint8_t *)malloc(nnew > 0 ? nnew : 1);
        uint8_t *state2 = (uint8_t *)malloc(nnew > 0 ? nnew : 1);
        int32_t *gslot2 = NULL;
        int gw = 2 * r->num_blocks;
        if (gw > 0) gslot2 = (int32_t *)malloc((size_t)(nnew > 0 ? nnew : 1) * sizeof(int32_t));
        int64_t k = 0;
        for (int64_t i = 0; i < n; i++) {
            if (out[i].dead) continue;
            id2[k] = r->id[i];
            cell2[k] = (out[i].move_to >= 0) ? out[i].move_to : r->cell[i];
            birth2[k] = r->birth[i]; age2[k] = r->age[i]; lastb2[k] = r->lastb[i];
            gender2[k] = r->gender[i]; state2[k] = r->state[i];
            if (gw > 0) gslot2[k] = r->gslot[i];
            k++;
        }
        /* newborns' genome slots: slots freed by earlier steps' deaths, then
         * unused ones; this step's deaths free theirs after the births, so a
         * newborn never takes a parent's slot of the same step */
        if (gw > 0) {
            reserve_slots(r, r->ghwm + nb);
            for (int64_t b = 0; b < nb; b++) {
                gslot2[nsurv + b] = (b < r->nfree) ? r->gfree[r->nfree - 1 - b] : (int32_t)(r->ghwm + (b - r->nfree));
            }
            if (nb > r->nfree) {
                r->ghwm += nb - r->nfree;
                r->nfree = 0;
            } else {
                r->nfree -= nb;
            }
        }
        if (r->log_births) {
            if (r->blog_n + nb > r->blog_cap) {
                int64_t cap = r->blog_cap ? r->blog_cap : 1024;
                while (cap < r->blog_n + nb) cap *= 2;
                r->blog = (int64_t *)realloc(r->blog, cap * 3 * sizeof(int64_t));
                r->blog_cap = cap;
            }
        }
#pragma omp parallel for schedule(static)
        for (int64_t b = 0; b < nb; b++) {
            int64_t m = mom[b];
            int64_t f = out[m].mate;
            int64_t kk = nsurv + b;
            stream_t s = { r->seed, (uint32_t)r->step, r->id[m], QHG_STREAM_BIRTH, 0 };
            /* SPopulation::createAgentAtIndex / resetAgent (core/SPopulation.cpp:880-918) */
            uint8_t g = (uint8_t)(2 * u2d(next_draw(&s)));
            id2[kk] = r->next_id + b;
            cell2[kk] = r->cell[m];
            birth2[kk] = fT;
            age2[kk] = 0.0f;
            lastb2[kk] = 0.0f;
            gender2[kk] = g;
            state2[kk] = (g == 0) ? LS_FERTILE : LS_ALIVE;
            if (gw > 0) {
                make_genome(r, r->genome + (size_t)gslot2[kk] * gw, r->genome + (size_t)r->gslot[m] * gw,
                            r->genome + (size_t)r->gslot[f] * gw, &s);
            }
            if (r->log_births) {
                r->blog[(r->blog_n + b) * 3 + 0] = r->next_id + b;
                r->blog[(r->blog_n + b) * 3 + 1] = r->id[m];
                r->blog[(r->blog_n + b) * 3 + 2] = r->id[f];
            }
        }
        if (r->log_births) r->blog_n += nb;
        r->next_id += nb;
        if (gw > 0) {
            for (int64_t i = 0; i < n; i++) {
                if (out[i].dead) r->gfree[r->nfree++] = r->gslot[i];
            }
        }
        free(mom);
        free(out);
        free(r->id); free(r->cell); free(r->birth); free(r->age); free(r->lastb);
        free(r->gender); free(r->state); free(r->gslot);
        r->id = id2; r->cell = cell2; r->birth = birth2; r->age = age2; r->lastb = lastb2;
        r->gender = gender2; r->state = state2; r->gslot = gslot2;
        r->n = nnew;
        r->cap = nnew > 0 ? nnew : 1;
        recount(r);
        if (stats_out != NULL) {
            stats_out[st * 4 + 0] = (uint64_t)nnew;
            stats_out[st * 4 + 1] = (uint64_t)nb;
            stats_out[st * 4 + 2] = nDeaths;
            stats_out[st * 4 + 3] = nMoves;
        }
        r->step++;
    }
    (void)ensure_stats;
    return 0;
}

int64_t qo_num_agents(const qo_run *r) { return r->n; }
int32_t qo_current_step(const qo_run *r) { return r->step; }
int64_t qo_next_id(const qo_run *r) { return r->next_id; }
void qo_set_next_id(qo_run *r, int64_t next_id) { r->next_id = next_id; }

int qo_get_agents(const qo_run *r, int64_t *id, int32_t *cell, float *birth, float *age, float *lastb,
                  uint8_t *gender, uint8_t *state, uint64_t *genome) {
    int64_t n = r->n;
    memcpy(id, r->id, n * sizeof(int64_t));
    memcpy(cell, r->cell, n * sizeof(int32_t));
    memcpy(birth, r->birth, n * sizeof(float));
    memcpy(age, r->age, n * sizeof(float));
    memcpy(lastb, r->lastb, n * sizeof(float));
    memcpy(gender, r->gender, n);
    memcpy(state, r->state, n);
    if (genome != NULL && r->num_blocks > 0) {
        const int gw = 2 * r->num_blocks;
#pragma omp parallel for schedule(static)
        for (int64_t k = 0; k < n; k++) {
            memcpy(genome + (size_t)k * gw, r->genome + (size_t)r->gslot[k] * gw, gw * sizeof(uint64_t));
        }
    }
    return 0;
}

int qo_get_counts(const qo_run *r, uint32_t *counts) {
    memcpy(counts, r->count, r->C * sizeof(uint32_t));
    return 0;
}

int64_t qo_num_logged_births(const qo_run *r) { return r->blog_n; }

int qo_get_birth_log(const qo_run *r, int64_t *baby, int64_t *mother, int64_t *father) {
    for (int64_t i = 0; i < r->blog_n; i++) {
        baby[i] = r->blog[i * 3];
        mother[i] = r->blog[i * 3 + 1];
        father[i] = r->blog[i * 3 + 2];
    }
    return 0;
}

int qo_binomial_table(const qo_run *r, double *out, int cap) {
    int n = r->n_bino < cap ? r->n_bino : cap;
    for (int i = 0; i < n; i++) out[i] = r->bino[i];
    return r->n_bino;
}

void qo_set_log_births(qo_run *r, int on) { r->log_births = on; }

/* MoveStats with the given mode (0 first, 1 min, 2 last) and cell
 * coordinates (lon/lat in degrees on a sphere of radius R, or x/y on a plane
 * when cartesian); initialised from the loaded agents, if any */
int qo_move_stats_enable(qo_run *r, int mode, const double *lon, const double *lat, double R, int cartesian) {
    if (mode < 0 || mode > 2) return -1;
    const size_t C = (size_t)r->C;
    if (r->ms_lon == NULL) {
        r->ms_lon = (double *)malloc(C * sizeof(double)); r->ms_lat = (double *)malloc(C * sizeof(double));
        r->ms_hops = (int32_t *)malloc(C * sizeof(int32_t)); r->ms_thops = (int32_t *)malloc(C * sizeof(int32_t));
        r->ms_dist = (double *)malloc(C * sizeof(double)); r->ms_time = (double *)malloc(C * sizeof(double));
        r->ms_tdist = (double *)malloc(C * sizeof(double)); r->ms_ttime = (double *)malloc(C * sizeof(double));
        r->ms_changed = (uint8_t *)malloc(C);
    }
    memcpy(r->ms_lon, lon, C * sizeof(double));
    memcpy(r->ms_lat, lat, C * sizeof(double));
    r->ms_R = R;
    r->ms_cart = cartesian;
    r->ms_mode = mode;
    ms_init(r);
    return 0;
}

int qo_move_stats(const qo_run *r, int32_t *hops, double *dist, double *time) {
    if (r->ms_mode < 0) return -1;
    memcpy(hops, r->ms_hops, (size_t)r->C * sizeof(int32_t));
    memcpy(dist, r->ms_dist, (size_t)r->C * sizeof(double));
    memcpy(time, r->ms_time, (size_t)r->C * sizeof(double));
    return 0;
}

/* A new K per cell from the next step on: VerhulstVarK's rates are computed
 * from K at each step's initialize (actions/LinearBirth.cpp:90-112,
 * actions/LinearDeath.cpp:92-122).  Unless weights were given, WeightedMove's
 * weights follow K (an always-updating SingleEvaluator). */
int qo_set_capacity(qo_run *r, const double *K) {
    memcpy(r->K, K, (size_t)r->C * sizeof(double));
    if (!r->w_given) weights_from_K(r);
    return 0;
}

/* WeightedMove's cumulative weights as a MultiEvaluator or SingleEvaluator
 * leaves them (C x 7, actions/MultiEvaluator.cpp:221-255), from the next
 * step on; they no longer follow K. */
int qo_set_move_weights(qo_run *r, const double *W) {
    memcpy(r->W, W, (size_t)r->C * 7 * sizeof(double));
    r->w_given = 1;
    return 0;
}

/* Geography::m_abIce per cell (nonzero: ice), from the next step on;
 * WeightedMove refuses moves into ice cells (actions/WeightedMove.cpp:91)
 * and the SingleEvaluator over K gives them weight 0
 * (actions/SingleEvaluator.cpp:183-202).  NULL removes the Geography's ice. */
int qo_set_ice(qo_run *r, const uint8_t *ice) {
    if (ice == NULL) {
        free(r->ice);
        r->ice = NULL;
    } else {
        if (r->ice == NULL) r->ice = (uint8_t *)malloc((size_t)r->C);
        if (r->ice == NULL) return -1;
        memcpy(r->ice, ice, (size_t)r->C);
    }
    /* weights that follow K give ice cells weight 0 */
    if (!r->w_given) weights_from_K(r);
    return 0;
}

void qo_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int qo_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void qo_destroy(qo_run *r) {
    if (r == NULL) return;
    free(r->nbr); free(r->nnbr); free(r->K); free(r->W); free(r->count); free(r->B); free(r->D); free(r->ice);
    free(r->ms_lon); free(r->ms_lat); free(r->ms_hops); free(r->ms_thops); free(r->ms_dist);
    free(r->ms_time); free(r->ms_tdist); free(r->ms_ttime); free(r->ms_changed);
    free(r->id); free(r->cell); free(r->birth); free(r->age); free(r->lastb); free(r->gender);
    free(r->state); free(r->genome); free(r->gslot); free(r->gfree); free(r->bino); free(r->blog); free(r->stats);
    free(r);
}
