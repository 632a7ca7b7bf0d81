// Step kernels of libqhg_gpu.so (sm_103a).
//
// Agents live in device memory as a structure of arrays sorted by cell:
// cell c owns rows [cell_start[c], cell_start[c+1]).  One step is three
// kernels (plus the genome kernel with genetics):
//
//   k_actions   one warp per non-empty cell.  Computes the cell's Verhulst
//               thresholds, pairs its FERTILE agents (RandomPair), runs every
//               action on every agent of the cell and writes one outcome
//               byte per agent (dead / stays / moves to neighbour slot k,
//               gives birth, new fertility), per-cell class counts, and for
//               each mother the father's row and her birth rank by ID.
//   k_cell_scan one pass over all cells with a decoupled look-back scan:
//               new per-cell counts (stayers + movers in + births), new
//               cell_start, output bases of every (cell, class), birth
//               numbering and the next step's list of non-empty cells.
//   k_scatter   one warp per old non-empty cell: stable ranks per class by
//               warp ballots, every survivor and newborn written to its row
//               of the next table.  The last CTA commits the run state.
//
// The reference runs these as SPopulation::initializeStep / doActions /
// finalizeStep (core/SPopulation.cpp:394-577, 596-724, 1058-1092, 509-536).
#include <cstdint>
#include <cuda_runtime.h>

#include "qhg_device.cuh"

namespace qhg {

#define FULL_MASK 0xffffffffu

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__device__ __forceinline__ uint32_t pick4(const Draw4 &d, uint32_t k) {
    uint32_t a = (k & 1u) ? d.v[1] : d.v[0];
    uint32_t b = (k & 1u) ? d.v[3] : d.v[2];
    return (k & 2u) ? b : a;
}

// draws of one agent in one step: the per-agent action stream, caching the
// last Philox block
struct AgentDraws {
    uint64_t seed;
    int64_t id;
    uint32_t step;
    uint32_t blk;
    Draw4 d;
    __device__ __forceinline__ void init(uint64_t s, uint32_t st, int64_t i) {
        seed = s; step = st; id = i; blk = 0xffffffffu;
    }
    __device__ __forceinline__ uint32_t get(uint32_t k) {
        uint32_t b = kStreamActions + (k >> 2);
        if (b != blk) {
            d = draw_block(seed, step, id, b);
            blk = b;
        }
        return pick4(d, k & 3u);
    }
};

// position of the k-th (0-based) set bit of z; the bit must exist
__device__ __forceinline__ int select_bit(uint32_t z, int k) {
    int pos = 0;
    int c = __popc(z & 0xffffu);
    if (k >= c) { k -= c; pos += 16; z >>= 16; }
    c = __popc(z & 0xffu);
    if (k >= c) { k -= c; pos += 8; z >>= 8; }
    c = __popc(z & 0xfu);
    if (k >= c) { k -= c; pos += 4; z >>= 4; }
    c = __popc(z & 0x3u);
    if (k >= c) { k -= c; pos += 2; z >>= 2; }
    c = (int)(z & 1u);
    if (k >= c) { pos += 1; }
    return pos;
}

__device__ __forceinline__ void set_error(RunState *rs, uint32_t code, uint32_t info) {
    if (atomicCAS(&rs->error, 0u, code) == 0u) {
        rs->error_info = info;
    }
}

// u < thr  <=>  u / 2^32 < x   for a double x (the reference's wrandd() < x)
__device__ __forceinline__ uint64_t prob_threshold(double x) {
    if (!(x > 0.0)) return 0ull;
    double y = __dmul_rn(x, 4294967296.0);
    if (y >= 4294967296.0) return 4294967296ull;
    return (uint64_t)ceil(y);
}

struct WarpSmem {
    uint64_t fid[kMaxCell];     // FERTILE ids: females from the front, males from the back
    uint16_t floc[kMaxCell];    // their rows within the cell
    uint16_t srt[kMaxCell];     // sorted order (females front, males back)
    int16_t mate[kMaxCell];     // mate's row within the cell, -1 none
    uint16_t pick[kMaxCell];    // per pairing: chosen member of the larger side
    uint8_t bfl[kMaxCell];      // gives birth this step
    uint32_t taken[kMaxCell / 32];
    uint64_t thr[kMaxActions][2];  // Verhulst: birth (or birth-death) and death thresholds
    int32_t thr_kind[kMaxActions]; // 0 none, 1 birth, 2 death by negative birth rate
};

// ------------------------------------------------------------------ actions
__global__ void __launch_bounds__(kWarpsPerCta * 32)
k_actions(const StepConst P, RunState *__restrict__ rs,
          const uint32_t *__restrict__ cell_start, const uint32_t *__restrict__ nonempty,
          const int64_t *__restrict__ id, const float *__restrict__ birth,
          const float *__restrict__ age, const float *__restrict__ lastb,
          const uint8_t *__restrict__ meta,
          const int32_t *__restrict__ nbr, const uint8_t *__restrict__ nnbr,
          const double *__restrict__ Kc, const uint64_t *__restrict__ wthr,
          const uint8_t *__restrict__ wflag,
          uint8_t *__restrict__ outc, int32_t *__restrict__ father, uint16_t *__restrict__ brank,
          uint32_t *__restrict__ clsc) {
    __shared__ WarpSmem smem[kWarpsPerCta];
    if (rs->error != 0u) return;   // an earlier kernel failed: keep the state
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    WarpSmem &S = smem[warp];
    const uint32_t lt = lanemask_lt();
    const int32_t step = rs->step;
    const float fT = (float)step;
    const uint32_t n_ne = rs->n_nonempty;
    uint32_t cnt_births = 0, cnt_deaths = 0, cnt_moves = 0;

    for (uint32_t w = blockIdx.x * kWarpsPerCta + warp; w < n_ne; w += gridDim.x * kWarpsPerCta) {
        const int c = (int)nonempty[w];
        const uint32_t s = cell_start[c];
        const int n = (int)(cell_start[c + 1] - s);
        if (n > kMaxCell) {
            if (lane == 0) set_error(rs, kErrCellTooLarge, (uint32_t)c);
            continue;
        }
        // ---- per-cell rates (LinearBirth/LinearDeath::initialize)
        if (lane == 0) {
            for (int a = 0; a < P.n_act; a++) {
                const ActionConst &A = P.act[a];
                if (A.type != kVerhulst && A.type != kVerhulstVarK) continue;
                double B, D;
                double K = (A.type == kVerhulst) ? A.K : Kc[c];
                if (A.type == kVerhulstVarK && K <= 0.0) {
                    B = 0.0;
                    D = 1.0;
                } else {
                    double r = __ddiv_rn((double)n, K);
                    B = __dadd_rn(A.b0, __dmul_rn(A.th_b0, r));
                    D = __dadd_rn(A.d0, __dmul_rn(A.th_d0, r));
                }
                int kind = 0;
                uint64_t tb = 0;
                if (B > 0.0) { kind = 1; tb = prob_threshold(B); }
                else if (B < 0.0) { kind = 2; tb = prob_threshold(-B); }
                S.thr_kind[a] = kind;
                S.thr[a][0] = tb;
                S.thr[a][1] = prob_threshold(D);
            }
        }
        // ---- pairing (RandomPair::findMates, members in ID order, keyed picks)
        int nF = 0, nM = 0;
        for (int b = 0; b < n; b += 32) {
            const int i = b + lane;
            const bool in = i < n;
            const uint8_t m = in ? meta[s + i] : (uint8_t)0;
            const bool fert = P.has_pair && in && (m & kMetaFertile);
            const bool fem = fert && !(m & kMetaGender);
            const bool mal = fert && (m & kMetaGender);
            const uint32_t bf = __ballot_sync(FULL_MASK, fem);
            const uint32_t bm = __ballot_sync(FULL_MASK, mal);
            if (fem) {
                const int p = nF + __popc(bf & lt);
                S.fid[p] = id[s + i];
                S.floc[p] = (uint16_t)i;
            }
            if (mal) {
                const int p = kMaxCell - 1 - (nM + __popc(bm & lt));
                S.fid[p] = id[s + i];
                S.floc[p] = (uint16_t)i;
            }
            nF += __popc(bf);
            nM += __popc(bm);
            if (in) {
                S.mate[i] = -1;
                S.bfl[i] = 0;
            }
        }
        __syncwarp();
        if (nF > 0 && nM > 0) {
            // rank sort by ID (IDs are unique)
            for (int j = lane; j < nF; j += 32) {
                const uint64_t x = S.fid[j];
                int r = 0;
                for (int t = 0; t < nF; t++) r += (S.fid[t] < x) ? 1 : 0;
                S.srt[r] = (uint16_t)j;
            }
            for (int j = lane; j < nM; j += 32) {
                const uint64_t x = S.fid[kMaxCell - 1 - j];
                int r = 0;
                for (int t = 0; t < nM; t++) r += (S.fid[kMaxCell - 1 - t] < x) ? 1 : 0;
                S.srt[kMaxCell - 1 - r] = (uint16_t)j;
            }
            __syncwarp();
            const bool femSmall = nF <= nM;
            const int nS = femSmall ? nF : nM;
            const int nL = femSmall ? nM : nF;
            // each pick draws from the pairing stream of the picking member
            for (int r = lane; r < nS; r += 32) {
                int64_t sid;
                if (femSmall) sid = (int64_t)S.fid[S.srt[r]];
                else sid = (int64_t)S.fid[kMaxCell - 1 - S.srt[kMaxCell - 1 - r]];
                const uint32_t u = draw_block(P.seed, (uint32_t)step, sid, kStreamPair).v[0];
                const uint32_t nRem = (uint32_t)(nL - r);
                S.pick[r] = (uint16_t)(((uint64_t)nRem * (uint64_t)u) >> 32);
            }
            __syncwarp();
            if (lane == 0) {
                const int nw = (nL + 31) >> 5;
                for (int q = 0; q < nw; q++) S.taken[q] = 0u;
                for (int r = 0; r < nS; r++) {
                    int k = S.pick[r];
                    int p = -1;
                    for (int q = 0; q < nw; q++) {
                        uint32_t valid = (q == nw - 1 && (nL & 31)) ? ((1u << (nL & 31)) - 1u) : FULL_MASK;
                        uint32_t z = ~S.taken[q] & valid;
                        int pc = __popc(z);
                        if (k < pc) {
                            int bit = select_bit(z, k);
                            S.taken[q] |= 1u << bit;
                            p = q * 32 + bit;
                            break;
                        }
                        k -= pc;
                    }
                    S.pick[r] = (uint16_t)p;
                }
            }
            __syncwarp();
            for (int r = lane; r < nS; r += 32) {
                const int pl = S.pick[r];
                if (pl >= nL) {   // cannot happen: every pick finds a free member
                    set_error(rs, kErrInternal, 1u);
                    continue;
                }
                int locS, locL;
                if (femSmall) {
                    locS = S.floc[S.srt[r]];
                    locL = S.floc[kMaxCell - 1 - S.srt[kMaxCell - 1 - pl]];
                } else {
                    locS = S.floc[kMaxCell - 1 - S.srt[kMaxCell - 1 - r]];
                    locL = S.floc[S.srt[pl]];
                }
                S.mate[locS] = (int16_t)locL;
                S.mate[locL] = (int16_t)locS;
            }
        }
        __syncwarp();
        // ---- actions on every agent (SPopulation::doActions)
        const int nn = nnbr[c];
        uint32_t cls_cnt[kCls];
#pragma unroll
        for (int k = 0; k < kCls; k++) cls_cnt[k] = 0;
        for (int b = 0; b < n; b += 32) {
            const int i = b + lane;
            const bool in = i < n;
            int cls = 0;
            bool bflag = false;
            if (in) {
                const uint32_t row = s + (uint32_t)i;
                const int64_t aid = id[row];
                const uint8_t m8 = meta[row];
                const float fb = birth[row];
                float fa = age[row];
                const float fl = lastb[row];
                const bool female = !(m8 & kMetaGender);
                bool fert = (m8 & kMetaFertile) != 0;
                bool alive = true;
                int dir = 0;
                AgentDraws dr;
                dr.init(P.seed, (uint32_t)step, aid);
                for (int a = 0; a < P.n_act && alive; a++) {
                    const ActionConst &A = P.act[a];
                    switch (A.type) {
                    case kGetOld:
                        fa = __fsub_rn(fT, fb);
                        break;
                    case kFertility:
                        if (female) fert = (fa > A.f0) && (fa < A.f1) && (__fsub_rn(fT, fl) > A.f2);
                        else fert = fa > A.f0;
                        break;
                    case kVerhulst:
                    case kVerhulstVarK: {
                        uint32_t k = A.window;
                        const int kind = S.thr_kind[a];
                        if (kind == 1) {
                            if (female && S.mate[i] >= 0) {
                                if ((uint64_t)dr.get(k++) < S.thr[a][0]) bflag = true;
                            }
                        } else if (kind == 2) {
                            if ((uint64_t)dr.get(k++) < S.thr[a][0]) alive = false;
                        }
                        if (alive) {
                            if ((uint64_t)dr.get(k) < S.thr[a][1]) alive = false;
                        }
                        if (!alive) cnt_deaths++;
                        break;
                    }
                    case kOldAgeDeath: {
                        fa = __fsub_rn(fT, fb);
                        bool die;
                        if (fa <= A.age_lo) {
                            die = false;
                        } else if (fa > A.age_hi) {
                            die = true;
                        } else {
                            const uint32_t u = dr.get(A.window);
                            double t = __dmul_rn(__dmul_rn(A.oad_w, (double)u), 2.3283064365386962890625e-10);
                            double thr = __dadd_rn(A.oad_M, __dadd_rn(A.oad_a, t));
                            die = (double)fa > thr;
                        }
                        if (die) { alive = false; cnt_deaths++; }
                        break;
                    }
                    case kRandomMove: {
                        if ((uint64_t)dr.get(A.window) < A.pthr) {
                            const uint32_t u2 = dr.get(A.window + 1);
                            const int d = (int)(((uint64_t)(nn + 1) * (uint64_t)u2) >> 32);
                            if (d > 0) {
                                const int to = nbr[c * 6 + d - 1];
                                if (to >= 0) { dir = d; cnt_moves++; }
                            }
                        }
                        break;
                    }
                    case kWeightedMove: {
                        if ((uint64_t)dr.get(A.window) < A.pthr) {
                            const uint32_t u2 = dr.get(A.window + 1);
                            int d;
                            if (wflag[c] & 1u) {
                                d = (int)(((uint64_t)(nn + 1) * (uint64_t)u2) >> 32);
                            } else {
                                d = 0;
                                for (int j = 0; j < nn; j++) d += (wthr[c * 6 + j] <= (uint64_t)u2) ? 1 : 0;
                            }
                            if (d > 0) {
                                const int to = nbr[c * 6 + d - 1];
                                if (to >= 0) { dir = d; cnt_moves++; }
                            }
                        }
                        break;
                    }
                    default:
                        break;
                    }
                }
                cls = alive ? (1 + dir) : 0;
                const uint8_t code = (uint8_t)(cls | (bflag ? kOutBirth : 0) | (fert ? kOutFertile : 0) |
                                               ((m8 & kMetaGender) ? kOutGender : 0));
                outc[row] = code;
                if (bflag) {
                    father[row] = (int32_t)(s + (uint32_t)S.mate[i]);
                    S.bfl[i] = 1;
                    cnt_births++;
                }
            }
#pragma unroll
            for (int k = 1; k < kCls; k++) cls_cnt[k - 1] += __popc(__ballot_sync(FULL_MASK, in && cls == k));
            cls_cnt[kCls - 1] += __popc(__ballot_sync(FULL_MASK, bflag));
        }
        __syncwarp();
        // ---- birth ranks by mother ID (births are numbered in (cell, mother ID) order)
        if (cls_cnt[kCls - 1] > 0) {
            int acc = 0;
            for (int b = 0; b < nF; b += 32) {
                const int r = b + lane;
                int loc = 0;
                bool mom = false;
                if (r < nF) {
                    loc = S.floc[S.srt[r]];
                    mom = S.bfl[loc] != 0;
                }
                const uint32_t mm = __ballot_sync(FULL_MASK, mom);
                if (mom) brank[s + loc] = (uint16_t)(acc + __popc(mm & lt));
                acc += __popc(mm);
            }
        }
        // ---- per-cell class counts
        uint32_t myv = 0;
#pragma unroll
        for (int k = 0; k < kCls; k++) myv = (lane == k) ? cls_cnt[k] : myv;
        if (lane < kCls) clsc[c * kCls + lane] = myv;
        __syncwarp();
    }
    // statistics of the step
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        cnt_births += __shfl_down_sync(FULL_MASK, cnt_births, o);
        cnt_deaths += __shfl_down_sync(FULL_MASK, cnt_deaths, o);
        cnt_moves += __shfl_down_sync(FULL_MASK, cnt_moves, o);
    }
    if (lane == 0 && (cnt_births | cnt_deaths | cnt_moves)) {
        unsigned long long *st = rs->stats[(uint32_t)step % kStatsRing];
        atomicAdd(&st[1], (unsigned long long)cnt_births);
        atomicAdd(&st[2], (unsigned long long)cnt_deaths);
        atomicAdd(&st[3], (unsigned long long)cnt_moves);
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

// look-back status words: (epoch << 2) | 1 aggregate ready, | 2 inclusive ready
__global__ void __launch_bounds__(kScanThreads)
k_cell_scan(const StepConst P, RunState *__restrict__ rs,
            const uint32_t *__restrict__ cell_start, const int32_t *__restrict__ nbr,
            const uint8_t *__restrict__ nnbr, const int32_t *__restrict__ rev,
            const uint32_t *__restrict__ clsc,
            uint32_t *__restrict__ new_start, uint32_t *__restrict__ sbase, uint32_t *__restrict__ bbase,
            uint32_t *__restrict__ bidbase, uint32_t *__restrict__ obase,
            uint32_t *__restrict__ new_nonempty,
            uint32_t *__restrict__ tile_flag, uint4 *__restrict__ tile_agg, uint4 *__restrict__ tile_incl) {
    __shared__ uint32_t s_tile;
    __shared__ ScanVal s_warp[kScanThreads / 32];
    __shared__ ScanVal s_prefix;
    if (rs->error != 0u) return;
    const int C = P.num_cells;
    const uint32_t ntiles = (uint32_t)((C + kScanTile - 1) / kScanTile);
    // flags of earlier steps carry older epochs; the host clears them when
    // the step counter is reset (upload, error recovery)
    const uint32_t epoch = ((uint32_t)rs->step + 1u) & 0x3fffffffu;
    if (threadIdx.x == 0) {
        uint32_t t = atomicAdd(&rs->scan_tiles_started, 1u);
        if (t == ntiles - 1) rs->scan_tiles_started = 0u;
        s_tile = t;
    }
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile >= ntiles) {   // stale tile counter: refuse rather than index past the status arrays
        if (threadIdx.x == 0) set_error(rs, kErrInternal, 2u);
        return;
    }
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int base = (int)tile * kScanTile + threadIdx.x * kScanItems;

    uint32_t nnew[kScanItems], stay[kScanItems], bth[kScanItems];
    ScanVal loc = {0u, 0u, 0u};
#pragma unroll
    for (int j = 0; j < kScanItems; j++) {
        const int d = base + j;
        nnew[j] = stay[j] = bth[j] = 0u;
        if (d < C) {
            const uint32_t nold = cell_start[d + 1] - cell_start[d];
            uint32_t st = 0, bt = 0;
            if (nold) {
                st = clsc[d * kCls + 0];
                bt = clsc[d * kCls + 7];
            }
            uint32_t mvin = 0;
            const int nn = nnbr[d];
            for (int q = 0; q < nn; q++) {
                const int sn = nbr[d * 6 + q];
                if (sn >= 0 && cell_start[sn + 1] != cell_start[sn]) {
                    mvin += clsc[sn * kCls + 1 + rev[d * 6 + q]];
                }
            }
            stay[j] = st;
            bth[j] = bt;
            nnew[j] = st + mvin + bt;
            loc.n += nnew[j];
            loc.b += bt;
            loc.ne += (nnew[j] > 0u) ? 1u : 0u;
        }
    }
    // block scan of the per-thread totals
    ScanVal inc = loc;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        ScanVal y = sv_shfl_up(inc, o);
        if (lane >= o) inc = sv_add(inc, y);
    }
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        ScanVal wv = (lane < kScanThreads / 32) ? s_warp[lane] : ScanVal{0u, 0u, 0u};
        ScanVal wi = wv;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            ScanVal y = sv_shfl_up(wi, o);
            if (lane >= o) wi = sv_add(wi, y);
        }
        if (lane < kScanThreads / 32) s_warp[lane] = ScanVal{wi.n - wv.n, wi.b - wv.b, wi.ne - wv.ne};
        // lane 7 holds the tile total
        const ScanVal total = {__shfl_sync(FULL_MASK, wi.n, kScanThreads / 32 - 1),
                               __shfl_sync(FULL_MASK, wi.b, kScanThreads / 32 - 1),
                               __shfl_sync(FULL_MASK, wi.ne, kScanThreads / 32 - 1)};
        if (lane == 0) {
            ScanVal excl = {0u, 0u, 0u};
            if (tile == 0) {
                tile_incl[tile] = make_uint4(total.n, total.b, total.ne, 0u);
                __threadfence();
                atomicExch(&tile_flag[tile], (epoch << 2) | 2u);
            } else {
                tile_agg[tile] = make_uint4(total.n, total.b, total.ne, 0u);
                __threadfence();
                atomicExch(&tile_flag[tile], (epoch << 2) | 1u);
                int t = (int)tile - 1;
                uint32_t spins = 0;
                while (t >= 0) {
                    const uint32_t f = atomicAdd(&tile_flag[t], 0u);
                    if ((f >> 2) != epoch || (f & 3u) == 0u) {
                        if (++spins > kSpinLimit) {
                            set_error(rs, kErrTimeout, tile);
                            break;
                        }
                        continue;
                    }
                    __threadfence();
                    const uint4 v = ((f & 3u) == 2u) ? __ldcg(&tile_incl[t]) : __ldcg(&tile_agg[t]);
                    excl.n += v.x; excl.b += v.y; excl.ne += v.z;
                    if ((f & 3u) == 2u) break;
                    t--;
                }
                tile_incl[tile] = make_uint4(excl.n + total.n, excl.b + total.b, excl.ne + total.ne, 0u);
                __threadfence();
                atomicExch(&tile_flag[tile], (epoch << 2) | 2u);
            }
            s_prefix = excl;
            if (tile == ntiles - 1) {
                const uint32_t tn = excl.n + total.n;
                rs->new_n_agents = tn;
                rs->new_n_nonempty = excl.ne + total.ne;
                rs->births = excl.b + total.b;
                new_start[C] = tn;
                if (tn > P.capacity) set_error(rs, kErrCapacity, tn);
            }
        }
    }
    __syncthreads();
    ScanVal pre = sv_add(s_prefix, s_warp[warp]);
    {
        ScanVal y = sv_shfl_up(inc, 1);
        if (lane >= 1) pre = sv_add(pre, y);
    }
#pragma unroll
    for (int j = 0; j < kScanItems; j++) {
        const int d = base + j;
        if (d < C) {
            new_start[d] = pre.n;
            sbase[d] = pre.n;
            bidbase[d] = pre.b;
            uint32_t run = pre.n + stay[j];
            const int nn = nnbr[d];
            for (int q = 0; q < nn; q++) {
                const int sn = nbr[d * 6 + q];
                if (sn >= 0 && cell_start[sn + 1] != cell_start[sn]) {
                    const int k = rev[d * 6 + q];
                    const uint32_t m = clsc[sn * kCls + 1 + k];
                    if (m) obase[sn * 6 + k] = run;
                    run += m;
                }
            }
            bbase[d] = run;
            if (nnew[j] > 0u) {
                new_nonempty[pre.ne] = (uint32_t)d;
                if (nnew[j] > (uint32_t)kMaxCell) set_error(rs, kErrCellTooLarge, (uint32_t)d);
            }
            pre.n += nnew[j];
            pre.b += bth[j];
            pre.ne += (nnew[j] > 0u) ? 1u : 0u;
        }
    }
}

// ----------------------------------------------------------------- scatter
__global__ void __launch_bounds__(kWarpsPerCta * 32)
k_scatter(const StepConst P, RunState *__restrict__ rs,
          const uint32_t *__restrict__ cell_start, const uint32_t *__restrict__ nonempty,
          const int64_t *__restrict__ id, const float *__restrict__ birth,
          const float *__restrict__ age, const float *__restrict__ lastb,
          const uint8_t *__restrict__ outc, const int32_t *__restrict__ father,
          const uint16_t *__restrict__ brank, const uint8_t *__restrict__ nnbr,
          const uint32_t *__restrict__ sbase, const uint32_t *__restrict__ bbase,
          const uint32_t *__restrict__ bidbase, const uint32_t *__restrict__ obase,
          int64_t *__restrict__ id2, float *__restrict__ birth2, float *__restrict__ age2,
          float *__restrict__ lastb2, uint8_t *__restrict__ meta2,
          int64_t *__restrict__ blog, uint64_t blog_cap) {
    if (rs->error != 0u) return;   // state stays as before the step
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const uint32_t lt = lanemask_lt();
    const int32_t step = rs->step;
    const float fT = (float)step;
    const int64_t next_id = rs->next_id;
    const uint64_t blog_base = rs->birth_log_n;
    const uint32_t n_ne = rs->n_nonempty;
    const uint32_t n_old = rs->n_agents;
    const uint32_t cap = P.capacity;
    for (uint32_t w = blockIdx.x * kWarpsPerCta + warp; w < n_ne; w += gridDim.x * kWarpsPerCta) {
        const int c = (int)nonempty[w];
        const uint32_t s = cell_start[c];
        const int n = (int)(cell_start[c + 1] - s);
        const uint32_t sb = sbase[c];
        const uint32_t bb = bbase[c];
        const uint32_t bid = bidbase[c];
        const int nn = nnbr[c];
        const uint32_t obv = (lane < nn) ? obase[c * 6 + lane] : 0u;
        uint32_t run[kCls - 1];
#pragma unroll
        for (int k = 0; k < kCls - 1; k++) run[k] = 0;
        for (int b = 0; b < n; b += 32) {
            const int i = b + lane;
            const bool in = i < n;
            const uint32_t row = s + (uint32_t)i;
            const uint8_t code = in ? outc[row] : (uint8_t)0;
            const int cls = code & 7;
            uint32_t r = 0;
#pragma unroll
            for (int k = 1; k < kCls; k++) {
                const uint32_t mk = __ballot_sync(FULL_MASK, in && cls == k);
                if (cls == k) r = run[k - 1] + __popc(mk & lt);
                run[k - 1] += __popc(mk);
            }
            const uint32_t mb = __shfl_sync(FULL_MASK, obv, (cls >= 2) ? (cls - 2) : 0);
            if (in && cls != 0) {
                const uint32_t dst = (cls == 1) ? (sb + r) : (mb + r);
                if (dst >= cap) {   // inconsistent bases: record, never write out of range
                    set_error(rs, kErrInternal, 3u);
                } else {
                    const float fb = birth[row];
                    id2[dst] = id[row];
                    birth2[dst] = fb;
                    lastb2[dst] = lastb[row];
                    age2[dst] = P.age_from_birth ? __fsub_rn(fT, fb) : age[row];
                    meta2[dst] = (uint8_t)(((code & kOutGender) ? kMetaGender : 0) |
                                           ((code & kOutFertile) ? kMetaFertile : 0));
                }
            }
            if (in && (code & kOutBirth)) {
                // SPopulation::createAgentAtIndex (core/SPopulation.cpp:880-900):
                // gender = (uchar)(2 * wrandd()), females start FERTILE
                const uint32_t rk = brank[row];
                const uint32_t dst = bb + rk;
                const int32_t fr = father[row];
                const bool ok = dst < cap && fr >= 0 && (uint32_t)fr < n_old;
                if (!ok) set_error(rs, kErrInternal, 4u);
                const int64_t mid = id[row];
                const uint32_t u = draw_block(P.seed, (uint32_t)step, mid, kStreamBirth).v[0];
                const uint8_t g = (uint8_t)(u >> 31);
                const int64_t baby = next_id + (int64_t)(bid + rk);
                if (ok) {
                    id2[dst] = baby;
                    birth2[dst] = fT;
                    lastb2[dst] = 0.0f;
                    age2[dst] = 0.0f;
                    meta2[dst] = (uint8_t)(g ? kMetaGender : kMetaFertile);
                    if (P.log_births) {
                        const uint64_t li = blog_base + (uint64_t)(bid + rk);
                        if (li < blog_cap) {
                            blog[li * 3 + 0] = baby;
                            blog[li * 3 + 1] = mid;
                            blog[li * 3 + 2] = id[fr];
                        }
                    }
                }
            }
        }
    }
    // the last CTA to finish commits the step
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const uint32_t done = atomicAdd(&rs->scatter_ctas_done, 1u);
        if (done == gridDim.x - 1) {
            __threadfence();
            rs->scatter_ctas_done = 0u;
            if (atomicAdd(&rs->error, 0u) != 0u) return;   // a CTA failed: keep the old table
            const uint32_t st = (uint32_t)rs->step;
            rs->stats[st % kStatsRing][0] = rs->new_n_agents;
            unsigned long long *nx = rs->stats[(st + 1u) % kStatsRing];
            nx[0] = 0ull; nx[1] = 0ull; nx[2] = 0ull; nx[3] = 0ull;
            rs->n_agents = rs->new_n_agents;
            rs->n_nonempty = rs->new_n_nonempty;
            rs->next_id += (int64_t)rs->births;
            rs->birth_log_n += rs->births;
            rs->step = (int32_t)(st + 1u);
            rs->scatter_ctas_done = 0u;
            __threadfence();
        }
    }
}

}  // namespace qhg

extern "C" int qhg_launch_step(const qhg::StepConst *P, qhg::RunState *rs, const qhg::StepBuffers *B,
                               int cell_grid, cudaStream_t stream) {
    using namespace qhg;
    const int C = P->num_cells;
    const int ntiles = (C + kScanTile - 1) / kScanTile;
    k_actions<<<cell_grid, kWarpsPerCta * 32, 0, stream>>>(
        *P, rs, B->cell_start, B->nonempty, B->id, B->birth, B->age, B->lastb, B->meta,
        B->nbr, B->nnbr, B->K, B->wthr, B->wflag, B->outc, B->father, B->brank, B->clsc);
    k_cell_scan<<<ntiles, kScanThreads, 0, stream>>>(
        *P, rs, B->cell_start, B->nbr, B->nnbr, B->rev, B->clsc, B->cell_start2, B->sbase, B->bbase,
        B->bidbase, B->obase, B->nonempty2, B->tile_flag, B->tile_agg, B->tile_incl);
    k_scatter<<<cell_grid, kWarpsPerCta * 32, 0, stream>>>(
        *P, rs, B->cell_start, B->nonempty, B->id, B->birth, B->age, B->lastb, B->outc, B->father,
        B->brank, B->nnbr, B->sbase, B->bbase, B->bidbase, B->obase, B->id2, B->birth2, B->age2,
        B->lastb2, B->meta2, B->blog, B->blog_cap);
    return (int)cudaGetLastError();
}

extern "C" int qhg_launch_step_timed(const qhg::StepConst *P, qhg::RunState *rs, const qhg::StepBuffers *B,
                                     int cell_grid, cudaStream_t stream, cudaEvent_t *ev) {
    using namespace qhg;
    const int C = P->num_cells;
    const int ntiles = (C + kScanTile - 1) / kScanTile;
    cudaEventRecord(ev[0], stream);
    k_actions<<<cell_grid, kWarpsPerCta * 32, 0, stream>>>(
        *P, rs, B->cell_start, B->nonempty, B->id, B->birth, B->age, B->lastb, B->meta,
        B->nbr, B->nnbr, B->K, B->wthr, B->wflag, B->outc, B->father, B->brank, B->clsc);
    cudaEventRecord(ev[1], stream);
    k_cell_scan<<<ntiles, kScanThreads, 0, stream>>>(
        *P, rs, B->cell_start, B->nbr, B->nnbr, B->rev, B->clsc, B->cell_start2, B->sbase, B->bbase,
        B->bidbase, B->obase, B->nonempty2, B->tile_flag, B->tile_agg, B->tile_incl);
    cudaEventRecord(ev[2], stream);
    k_scatter<<<cell_grid, kWarpsPerCta * 32, 0, stream>>>(
        *P, rs, B->cell_start, B->nonempty, B->id, B->birth, B->age, B->lastb, B->outc, B->father,
        B->brank, B->nnbr, B->sbase, B->bbase, B->bidbase, B->obase, B->id2, B->birth2, B->age2,
        B->lastb2, B->meta2, B->blog, B->blog_cap);
    cudaEventRecord(ev[3], stream);
    return (int)cudaGetLastError();
}
