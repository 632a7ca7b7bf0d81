/*
 * Oracle harness around the reference's own hot-path code.
 *
 * ORACLE / TEST INFRASTRUCTURE ONLY.  Built by oracle/ref/Makefile from the
 * reference sources (never copied into this repository) into two programs:
 *
 *   qhg_ref_well    the unmodified reference: WELL512 streams per OpenMP
 *                   thread, the reference's RandomPair, dead-slot recycling
 *                   and per-thread IDGen.  Used for the statistical (KS)
 *                   comparison and as the timed CPU baseline where it runs.
 *   qhg_ref_philox  the Philox test build: the same action classes, with
 *                   utils/WELL512.h replaced by oracle/ref/philox_well/WELL512.h
 *                   so that every draw is keyed by (seed, step, agent ID,
 *                   action); pairing sorts by agent ID and draws per pairing
 *                   member; births are ordered by (cell, mother ID) and get
 *                   sequential IDs.  Its output must match the C port oracle
 *                   and the CUDA path bit for bit.
 *
 * The step loop follows PopLooper::doStep (core/PopLooper.cpp:166-200):
 * initializeStep -> doActions per priority level -> finalizeStep.
 * The population mirrors tut_SexualPop / FlatExpPop
 * (populations/tut_SexualPop.cpp:24-43, populations/FlatExpPop.cpp:32-91):
 * an agent with age, last-birth time and mate index, and newborns with
 * age 0 and last birth 0 (populations/tut_SexualPop.cpp makePopSpecificOffspring).
 *
 * File formats are described in oracle/refsim_io.py.
 */
#include <omp.h>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <vector>
#include <algorithm>
#include <string>

#include "SPopulation.cpp"
#include "LayerBuf.cpp"
#include "LayerArrBuf.cpp"
#include "Prioritizer.cpp"
#include "Action.cpp"
#include "GetOld.cpp"
#include "Fertility.cpp"
#include "VerhulstVarK.cpp"
#include "OldAgeDeath.cpp"
#include "ATanDeath.cpp"
#include "RandomMove.cpp"
#include "WeightedMove.cpp"
#include "SingleEvaluator.cpp"
#include "RandomPair.cpp"
#include "MoveStats.cpp"
#include "BitGeneUtils.h"
#include "BinomialDist.h"
#include "Genetics.cpp"
#include "GenomeCreator.cpp"
#include "SequenceIOUtils.cpp"

#ifdef QHG_PHILOX_TEST_BUILD
thread_local QhgDrawContext g_qhgDrawCtx = {0, 0, 0, 0, 0, 0, 0};
unsigned long g_qhgDrawErrors = 0;
#endif

/* action type codes shared with oracle/refsim_io.py and include/qhg_gpu.h */
enum {
    ACT_GETOLD = 0, ACT_FERTILITY = 1, ACT_RANDOMPAIR = 2, ACT_VERHULST = 3,
    ACT_VERHULSTVARK = 4, ACT_OLDAGEDEATH = 5, ACT_RANDOMMOVE = 6, ACT_WEIGHTEDMOVE = 7,
    ACT_ATANDEATH = 8
};
/* the crossover mode that draws a Poisson(1) number of breakpoints per parent */
static const int CROSSOVER_POISSON1 = -100;

struct RefAgent : Agent {
    float m_fAge;
    float m_fLastBirth;
    int   m_iMateIndex;
};

static int g_curStep = 0;
static uint64_t g_seed = 0;

/* Poisson(1) inverse-CDF thresholds: floor(P(K <= k) * 2^32), k = 0..15,
 * computed exactly with rational arithmetic.  The same table is used by the
 * C port oracle and by the CUDA library. */
static const uint32_t POISSON1_CDF32[16] = {
    1580030168u, 3160060337u, 3950075421u, 4213413783u, 4279248373u,
    4292415291u, 4294609777u, 4294923276u, 4294962463u, 4294966817u,
    4294967252u, 4294967292u, 4294967295u, 4294967295u, 4294967295u,
    4294967295u
};

static int poissonFromDraw(uint32_t u) {
    int k = 0;
    while (k < 16 && u >= POISSON1_CDF32[k]) {
        k++;
    }
    return k;
}

/* ---------------------------------------------------------------------- */
#ifdef QHG_PHILOX_TEST_BUILD
/*
 * Keyed pairing for the test build.  Same rule as RandomPair::findMates
 * (actions/RandomPair.cpp:146-270): per cell, the FERTILE members of the
 * smaller sex are taken in order and each picks the wrandr(0, n)-th
 * still-unpaired member of the other sex.  Differences that make the result
 * layout-independent: members are ordered by agent ID instead of slot
 * index, and the draw of each pick is keyed by the picking member's ID.
 */
template<typename T>
class KeyedPair : public Action<T> {
public:
    KeyedPair(SPopulation<T> *pPop, SCellGrid *pCG, WELL512 **apWELL)
        : Action<T>(pPop, pCG, ATTR_RANDPAIR_NAME, ""), m_apWELL(apWELL) {}

    virtual int initialize(float fT) {
        int iFirst = this->m_pPop->getFirstAgentIndex();
        int iLast  = this->m_pPop->getLastAgentIndex();
        int C = (int)this->m_pCG->m_iNumCells;
        std::vector<std::vector<std::pair<idtype,int> > > vF(C), vM(C);
        if (iFirst != LBController::NIL) {
            for (int iA = iFirst; iA <= iLast; iA++) {
                this->m_pPop->m_aAgents[iA].m_iMateIndex = -3;
            }
            for (int iA = iFirst; iA <= iLast; iA++) {
                T *pA = &(this->m_pPop->m_aAgents[iA]);
                if ((pA->m_iLifeState > 0) && (pA->m_iLifeState == LIFE_STATE_FERTILE)) {
                    if (pA->m_iGender == 0) {
                        vF[pA->m_iCellIndex].push_back(std::make_pair(pA->m_ulID, iA));
                    } else if (pA->m_iGender == 1) {
                        vM[pA->m_iCellIndex].push_back(std::make_pair(pA->m_ulID, iA));
                    }
                }
            }
        }
#pragma omp parallel for schedule(dynamic, 64)
        for (int iC = 0; iC < C; iC++) {
            std::vector<std::pair<idtype,int> > &F = vF[iC];
            std::vector<std::pair<idtype,int> > &M = vM[iC];
            int nF = (int)F.size();
            int nM = (int)M.size();
            if ((nF > 0) && (nM > 0)) {
                std::sort(F.begin(), F.end());
                std::sort(M.begin(), M.end());
                bool bFewerF = (nF <= nM);
                std::vector<std::pair<idtype,int> > &S = bFewerF ? F : M;
                std::vector<std::pair<idtype,int> > &L = bFewerF ? M : F;
                int nS = (int)S.size();
                int nRem = (int)L.size();
                std::vector<bool> taken(L.size(), false);
                int iT = omp_get_thread_num();
                for (int j = 0; (j < nS) && (nRem > 0); j++) {
                    g_qhgDrawCtx = {g_seed, (uint32_t)g_curStep, S[j].first, QHG_STREAM_PAIR, 0, 1, 1};
                    int iChoose = (int)(m_apWELL[iT]->wrandr(0, nRem));
                    g_qhgDrawCtx.active = 0;
                    int iSearch = -1;
                    int iL = -1;
                    while (iSearch < iChoose) {
                        iL++;
                        if (!taken[iL]) {
                            iSearch++;
                        }
                    }
                    taken[iL] = true;
                    this->m_pPop->m_aAgents[S[j].second].m_iMateIndex = L[iL].second;
                    this->m_pPop->m_aAgents[L[iL].second].m_iMateIndex = S[j].second;
                    nRem--;
                }
            }
        }
        return 0;
    }
protected:
    WELL512 **m_apWELL;
};
#endif

/* ---------------------------------------------------------------------- */
/* Genetics with access to init() (protected in actions/Genetics.h) */
/* the reference's MoveStats with its per-cell results readable */
class HarnessMoveStats : public MoveStats<RefAgent> {
public:
    HarnessMoveStats(SPopulation<RefAgent> *pPop, SCellGrid *pCG) : MoveStats<RefAgent>(pPop, pCG, "") {}
    const int *hops() const { return this->m_aiHops; }
    const double *dist() const { return this->m_adDist; }
    const double *time() const { return this->m_adTime; }
};

class HarnessGenetics : public Genetics<RefAgent, BitGeneUtils> {
public:
    HarnessGenetics(SPopulation<RefAgent> *pPop, SCellGrid *pCG, LBController *pAC,
                    std::vector<int> *pvDead, WELL512 **apWELL)
        : Genetics<RefAgent, BitGeneUtils>(pPop, pCG, "", pAC, pvDead, apWELL) {}
    int doInit() { return this->init(); }
    int numCrossOvers() { return this->m_iNumCrossOvers; }
    double mutationRate() { return this->m_dMutationRate; }
    BinomialDist *bdist(int iT) { return this->m_pBDist[iT]; }
};

struct ActionSpec {
    uint32_t type;
    uint32_t prio;
    double   p[4];
};

/* ---------------------------------------------------------------------- */
class OraclePop : public SPopulation<RefAgent> {
public:
    OraclePop(SCellGrid *pCG, int iLayerSize, IDGen **apIDG, uint32_t *aulState, uint *aiSeeds)
        : SPopulation<RefAgent>(pCG, NULL, iLayerSize, apIDG, aulState, aiSeeds),
          m_pGenetics(NULL), m_adK(NULL), m_adWeights(NULL), m_iNextID(0),
          m_iGenomeSize(0), m_iNumBlocks(0), m_iCrossMode(0) {
        m_sSpeciesName = "oracle";
        m_sClassName   = "OraclePop";
    }

    virtual ~OraclePop() {
        for (size_t i = 0; i < m_vOwned.size(); i++) {
            delete m_vOwned[i];
        }
        delete[] m_adK;
        delete[] m_adWeights;
        for (size_t i = 0; i < m_vTemp.size(); i++) {
            delete[] m_vTemp[i];
        }
    }

    /* adGivenW: WeightedMove's cumulative weights as given (C x 7, what a
     * MultiEvaluator leaves, actions/MultiEvaluator.cpp:221-255), or NULL for
     * weights from K through an always-updating SingleEvaluator */
    /* iMoveStatsMode >= 0: a MoveStats action with that mode (the grid must
     * carry a Geography) */
    int setup(const std::vector<ActionSpec> &vSpecs, const double *adK,
              int iGenomeSize, int iNumCrossOvers, double dMutRate, const double *adGivenW,
              int iMoveStatsMode) {
        int C = (int)m_pCG->m_iNumCells;
        m_adK = new double[C];
        memcpy(m_adK, adK, C*sizeof(double));
        m_adWeights = new double[(size_t)C*(m_pCG->m_iConnectivity+1)];
        memset(m_adWeights, 0, (size_t)C*(m_pCG->m_iConnectivity+1)*sizeof(double));
        if (adGivenW != NULL) {
            memcpy(m_adWeights, adGivenW, (size_t)C*(m_pCG->m_iConnectivity+1)*sizeof(double));
        }

        int iResult = 0;
        for (size_t i = 0; (iResult == 0) && (i < vSpecs.size()); i++) {
            const ActionSpec &s = vSpecs[i];
            Action<RefAgent> *pA = NULL;
            ModuleComplex mc;
            char buf[64];
            switch (s.type) {
            case ACT_GETOLD:
                pA = new GetOld<RefAgent>(this, m_pCG, "");
                break;
            case ACT_FERTILITY:
                pA = new Fertility<RefAgent>(this, m_pCG, "");
                snprintf(buf, 64, "%.17g", s.p[0]); mc.addParam(ATTR_FERTILITY_MIN_AGE_NAME, buf);
                snprintf(buf, 64, "%.17g", s.p[1]); mc.addParam(ATTR_FERTILITY_MAX_AGE_NAME, buf);
                snprintf(buf, 64, "%.17g", s.p[2]); mc.addParam(ATTR_FERTILITY_INTERBIRTH_NAME, buf);
                break;
            case ACT_RANDOMPAIR:
#ifdef QHG_PHILOX_TEST_BUILD
                pA = new KeyedPair<RefAgent>(this, m_pCG, m_apWELL);
#else
                pA = new RandomPair<RefAgent>(this, m_pCG, "", m_apWELL);
#endif
                break;
            case ACT_VERHULST:
            case ACT_VERHULSTVARK: {
                /* a constant K > 0 gives the same rates through VerhulstVarK
                 * (actions/LinearBirth.cpp:97-108); Verhulst.cpp and
                 * VerhulstVarK.cpp cannot share one translation unit */
                double *adK = m_adK;
                if (s.type == ACT_VERHULST) {
                    adK = new double[C];
                    for (int c = 0; c < C; c++) adK[c] = s.p[3];
                    m_vTemp.push_back(adK);
                }
                pA = new VerhulstVarK<RefAgent>(this, m_pCG, "", m_apWELL, adK, 1);
                snprintf(buf, 64, "%.17g", s.p[0]); mc.addParam(ATTR_VERHULSTVARK_B0_NAME, buf);
                snprintf(buf, 64, "%.17g", s.p[1]); mc.addParam(ATTR_VERHULSTVARK_D0_NAME, buf);
                snprintf(buf, 64, "%.17g", s.p[2]); mc.addParam(ATTR_VERHULSTVARK_TURNOVER_NAME, buf);
                break;
            }
            case ACT_OLDAGEDEATH:
                pA = new OldAgeDeath<RefAgent>(this, m_pCG, "", m_apWELL);
                snprintf(buf, 64, "%.17g", s.p[0]); mc.addParam(ATTR_OLDAGEDEATH_MAXAGE_NAME, buf);
                snprintf(buf, 64, "%.17g", s.p[1]); mc.addParam(ATTR_OLDAGEDEATH_UNCERTAINTY_NAME, buf);
                break;
            case ACT_ATANDEATH:
                pA = new ATanDeath<RefAgent>(this, m_pCG, "", m_apWELL);
                snprintf(buf, 64, "%.17g", s.p[0]); mc.addParam(ATTR_ATANDEATH_MAXAGE_NAME, buf);
                snprintf(buf, 64, "%.17g", s.p[1]); mc.addParam(ATTR_ATANDEATH_RANGE_NAME, buf);
                snprintf(buf, 64, "%.17g", s.p[2]); mc.addParam(ATTR_ATANDEATH_SLOPE_NAME, buf);
                break;
            case ACT_RANDOMMOVE:
                pA = new RandomMove<RefAgent>(this, m_pCG, "", m_apWELL);
                snprintf(buf, 64, "%.17g", s.p[0]); mc.addParam(ATTR_RANDOMMOVE_PROB_NAME, buf);
                break;
            case ACT_WEIGHTEDMOVE: {
                /* weights: direct cell values K, cumulated over the
                 * neighbours (actions/SingleEvaluator.cpp:174-241) */
                if (adGivenW == NULL) {
                    SingleEvaluator<RefAgent> *pSE = new SingleEvaluator<RefAgent>(
                        this, m_pCG, "", m_adWeights, m_adK, "", true, EVENT_ID_NONE, true);
                    m_vOwned.push_back(pSE);
                    m_prio.addAction(pSE);
                    m_mPrioInfo[pSE->getActionName()] = (int)s.prio;
                }
                pA = new WeightedMove<RefAgent>(this, m_pCG, "", m_apWELL, m_adWeights);
                snprintf(buf, 64, "%.17g", s.p[0]); mc.addParam(ATTR_WEIGHTEDMOVE_PROB_NAME, buf);
                break;
            }
            default:
                fprintf(stderr, "unknown action type %u\n", s.type);
                iResult = -1;
            }
            if (pA != NULL) {
                if ((s.type != ACT_GETOLD) && (s.type != ACT_RANDOMPAIR)) {
                    if (pA->tryGetAttributes(&mc) != 0) {
                        fprintf(stderr, "tryGetAttributes failed for action type %u\n", s.type);
                        iResult = -1;
                    }
                }
                m_vOwned.push_back(pA);
                m_prio.addAction(pA);
                m_mPrioInfo[pA->getActionName()] = (int)s.prio;
                m_vSpecs.push_back(s);
                m_vSpecActions.push_back(pA);
            }
        }
        if ((iResult == 0) && (iMoveStatsMode >= 0)) {
            m_pMoveStats = new HarnessMoveStats(this, m_pCG);
            ModuleComplex mc;
            char buf[64];
            snprintf(buf, 64, "%d", iMoveStatsMode); mc.addParam(ATTR_MOVESTATS_MODE_NAME, buf);
            if (m_pMoveStats->tryGetAttributes(&mc) != 0) {
                fprintf(stderr, "MoveStats tryGetAttributes failed\n");
                iResult = -1;
            }
            m_vOwned.push_back(m_pMoveStats);
            m_prio.addAction(m_pMoveStats);
            m_mPrioInfo[m_pMoveStats->getActionName()] = 0;
        }
        if (iResult == 0) {
            iResult = setPrioList();
        }
        if ((iResult == 0) && (iGenomeSize > 0)) {
            m_iGenomeSize = iGenomeSize;
            m_iCrossMode  = iNumCrossOvers;
            m_pGenetics = new HarnessGenetics(this, m_pCG, m_pAgentController, &m_vMergedDeadList, m_apWELL);
            m_vOwned.push_back(m_pGenetics);
            ModuleComplex mc;
            char buf[64];
            snprintf(buf, 64, "%d", iGenomeSize); mc.addParam(ATTR_GENETICS_GENOME_SIZE, buf);
            /* the Poisson mode is driven by the harness below; the reference
             * object gets 1 so that it allocates its crossover buffers */
            snprintf(buf, 64, "%d", (iNumCrossOvers == CROSSOVER_POISSON1) ? 1 : iNumCrossOvers);
            mc.addParam(ATTR_GENETICS_NUM_CROSSOVER, buf);
            snprintf(buf, 64, "%.17g", dMutRate); mc.addParam(ATTR_GENETICS_MUTATION_RATE, buf);
            mc.addParam(ATTR_GENETICS_INITIAL_MUTS, "-1");  /* numeric code of "random"; genomes are loaded from the input */
            mc.addParam(ATTR_GENETICS_CREATE_NEW_GENOME, "0");
            mc.addParam(ATTR_GENETICS_BITS_PER_NUC, "1");
            if (m_pGenetics->tryGetAttributes(&mc) != 0) {
                fprintf(stderr, "Genetics tryGetAttributes failed\n");
                iResult = -1;
            } else {
                iResult = m_pGenetics->doInit();
            }
            m_iNumBlocks = m_pGenetics->getNumBlocks();
            m_pBDistPoisson = BinomialDist::create(dMutRate, 2*iGenomeSize, 1e-6);
            m_vTmp1.resize(2*m_iNumBlocks);
            m_vTmp2.resize(2*m_iNumBlocks);
        }
        computeWindows();
        return iResult;
    }

    /* draw windows of the agent actions, in execution order */
    void computeWindows() {
        std::set<uint> sPrios;
        m_prio.getPrios(sPrios);
        uint32_t w = 0;
        for (std::set<uint>::const_iterator it = sPrios.begin(); it != sPrios.end(); ++it) {
            for (uint j = 0; j < m_prio.getNumActionsForPrio(*it); j++) {
                Action<RefAgent> *pA = m_prio.getAction(*it, j);
                uint32_t n = 0;
                for (size_t k = 0; k < m_vSpecActions.size(); k++) {
                    if (m_vSpecActions[k] == pA) {
                        uint32_t t = m_vSpecs[k].type;
                        if ((t == ACT_VERHULST) || (t == ACT_VERHULSTVARK) || (t == ACT_RANDOMMOVE) || (t == ACT_WEIGHTEDMOVE)) {
                            n = 2;
                        } else if ((t == ACT_OLDAGEDEATH) || (t == ACT_ATANDEATH)) {
                            n = 1;
                        }
                    }
                }
                m_mWindowBase[pA] = w;
                m_mWindowSize[pA] = n;
                w += n;
            }
        }
    }

    /* a runtime edit, as QHG4 applies one (Prioritizer::modifyAttributes) */
    int modify(const std::string &sName, double dValue) {
        return m_prio.modifyAttributes(sName, dValue);
    }

    /* the deaths of FlatExpPop::updateEvent after a geography event
     * (populations/FlatExpPop.cpp:187-214): registerDeath for every live
     * agent in a flagged cell, the dead removed before the next step */
    void killInCells(const uint8_t *aucKill) {
        int iFirst = getFirstAgentIndex();
        if (iFirst != LBController::NIL) {
            int iLast = getLastAgentIndex();
            for (int iA = iFirst; iA <= iLast; iA++) {
                if ((m_aAgents[iA].m_iLifeState > LIFE_STATE_DEAD) && aucKill[m_aAgents[iA].m_iCellIndex]) {
                    registerDeath(m_aAgents[iA].m_iCellIndex, iA);
                }
            }
        }
        recycleDeadSpaceNew();
        updateTotal();
        updateNumAgentsPerCell();
        initListIdx();
    }

    /* a new K per cell, read by VerhulstVarK (and the SingleEvaluator) at
     * the next initializeStep, as when an environment event changes it */
    void setK(const double *adK) {
        memcpy(m_adK, adK, m_pCG->m_iNumCells*sizeof(double));
    }

    int loadAgents(uint32_t N, const int64_t *aiID, const int32_t *aiCell, const float *afBirth,
                   const float *afAge, const float *afLastB, const uint8_t *aiGender,
                   const uint8_t *aiState, const uint64_t *aulGenome) {
        int iStart = -1;
        if (N > 0) {
            iStart = m_pAgentController->reserveSpace2(N);
        }
        int64_t iMax = -1;
        for (uint32_t i = 0; i < N; i++) {
            int iA = iStart + (int)i;
            RefAgent &a = m_aAgents[iA];
            a.m_iLifeState = aiState[i];
            a.m_iCellIndex = aiCell[i];
            a.m_ulID       = aiID[i];
            a.m_ulCellID   = m_pCG->m_aCells[aiCell[i]].m_iGlobalID;
            a.m_fBirthTime = afBirth[i];
            a.m_iGender    = aiGender[i];
            a.m_fAge       = afAge[i];
            a.m_fLastBirth = afLastB[i];
            a.m_iMateIndex = -3;
            if (aiID[i] > iMax) iMax = aiID[i];
            if (m_pGenetics != NULL) {
                memcpy(m_pGenetics->getGenome(iA), aulGenome + (size_t)i*2*m_iNumBlocks,
                       2*m_iNumBlocks*sizeof(ulong));
            }
        }
        m_iNextID = iMax + 1;
        for (int t = 0; t < m_iNumThreads; t++) {
            m_apIDGen[t]->setBase(m_iNextID);
        }
        return 0;
    }

#ifdef QHG_PHILOX_TEST_BUILD
    /* SPopulation::doActions (core/SPopulation.cpp:554-577) with the draw
     * context of each (agent, action) set before execute() */
    virtual int doActions(uint iPrio, float fTime) {
        int iFirstAgent = getFirstAgentIndex();
        if (iFirstAgent != LBController::NIL) {
            int iLastAgent = getLastAgentIndex();
            for (uint iMethod = 0; iMethod < m_prio.getNumActionsForPrio(iPrio); iMethod++) {
                Action<RefAgent> *pA = m_prio.getAction(iPrio, iMethod);
                uint32_t wb = m_mWindowBase[pA];
                uint32_t ws = m_mWindowSize[pA];
#pragma omp parallel for
                for (int iAgent = iFirstAgent; iAgent <= iLastAgent; iAgent++) {
                    if (m_aAgents[iAgent].m_iLifeState > LIFE_STATE_DEAD) {
                        g_qhgDrawCtx = {g_seed, (uint32_t)g_curStep, m_aAgents[iAgent].m_ulID,
                                        QHG_STREAM_ACTIONS, wb, wb + ws, 1};
                        pA->execute(iAgent, fTime);
                        g_qhgDrawCtx.active = 0;
                    }
                }
            }
        }
        return 0;
    }

    /* replaces SPopulation::recycleDeadSpaceNew (core/SPopulation.cpp:596-724)
     * in the test build: births in (cell, mother ID) order with sequential
     * IDs; the slots of this step's dead are released after the births, so
     * newborns never overwrite a parent of the same step (the reference gets
     * the same guarantee by recycling dead slots one step late). */
    virtual int recycleDeadSpaceNew() {
        struct B { int cell; int mother; int father; idtype mid; };
        std::vector<B> vB;
        ulong iNumDeaths = 0;
        for (int t = 0; t < m_iNumThreads; t++) {
            std::vector<int> &v = *m_vBirthList[t];
            for (size_t i = 0; i + 2 < v.size(); i += 3) {
                B b = {v[i], v[i+1], v[i+2], m_aAgents[v[i+1]].m_ulID};
                vB.push_back(b);
            }
            iNumDeaths += m_vDeathList[t]->size();
        }
        std::sort(vB.begin(), vB.end(), [](const B &x, const B &y) {
            return (x.cell != y.cell) ? (x.cell < y.cell) : (x.mid < y.mid);
        });
        for (size_t r = 0; r < vB.size(); r++) {
            const B &b = vB[r];
            int iSlot = m_pAgentController->getFreeIndex();
            g_qhgDrawCtx = {g_seed, (uint32_t)g_curStep, b.mid, QHG_STREAM_BIRTH, 0, 1u << 20, 1};
            createAgentAtIndex(iSlot, b.cell);
            m_aAgents[iSlot].m_ulID = m_iNextID + (idtype)r;
            makePopSpecificOffspring(iSlot, b.mother, b.father);
            g_qhgDrawCtx.active = 0;
            m_vBirthLog.push_back(m_aAgents[iSlot].m_ulID);
            m_vBirthLog.push_back(b.mid);
            m_vBirthLog.push_back(m_aAgents[b.father].m_ulID);
        }
        m_iNextID += (idtype)vB.size();
        for (int t = 0; t < m_iNumThreads; t++) {
            std::vector<int> &v = *m_vDeathList[t];
            for (size_t i = 0; i < v.size(); i++) {
                m_pAgentController->deleteElement(v[i]);
            }
        }
        m_iNumBirths += vB.size();
        m_iNumDeaths += iNumDeaths;
        m_iStepBirths = vB.size();
        m_iStepDeaths = iNumDeaths;
        m_iNumPrevDeaths = 0;
        return 0;
    }
#else
    virtual int recycleDeadSpaceNew() {
        ulong iB = 0, iD = 0;
        for (int t = 0; t < m_iNumThreads; t++) {
            iB += m_vBirthList[t]->size() / 3;
            iD += m_vDeathList[t]->size();
        }
        m_iStepBirths = iB;
        m_iStepDeaths = iD;
        return SPopulation<RefAgent>::recycleDeadSpaceNew();
    }
#endif

    virtual int performMoves() {
        ulong iM = 0;
        for (int t = 0; t < m_iNumThreads; t++) {
            iM += m_vMoveList[t]->size() / 3;
        }
        m_iStepMoves = iM;
        return SPopulation<RefAgent>::performMoves();
    }

    /* newborn fields as in tut_SexualPop / FlatExpPop, plus genetics */
    virtual int makePopSpecificOffspring(int iAgent, int iMother, int iFather) {
        int iResult = 0;
        if (m_pGenetics != NULL) {
            if (m_iCrossMode == CROSSOVER_POISSON1) {
                iResult = makeOffspringPoisson(iAgent, iMother, iFather);
            } else {
                iResult = m_pGenetics->makeOffspring(iAgent, iMother, iFather);
            }
        }
        m_aAgents[iAgent].m_fAge = 0.0;
        m_aAgents[iAgent].m_fLastBirth = 0.0;
        m_aAgents[iAgent].m_iMateIndex = -3;
        return iResult;
    }

    /* Genetics::makeOffspring (actions/Genetics.cpp:285-337) with the number
     * of crossovers per parent drawn from Poisson(1) after the strand picks;
     * crossOver, mutateNucs and BinomialDist are the reference's. */
    int makeOffspringPoisson(int iBaby, int iMother, int iFather) {
        int iT = omp_get_thread_num();
        ulong *pBaby = m_pGenetics->getGenome(iBaby);
        ulong *pG1 = m_pGenetics->getGenome(iMother);
        ulong *pG2 = m_pGenetics->getGenome(iFather);
        memset(pBaby, 0, 2*m_iNumBlocks*sizeof(ulong));
        int i1 = (int)(2*1.0*m_apWELL[iT]->wrandd());
        int i2 = (int)(2*1.0*m_apWELL[iT]->wrandd());
        int nM = poissonFromDraw(m_apWELL[iT]->wrand());
        int nF = poissonFromDraw(m_apWELL[iT]->wrand());
        const ulong *pS1 = pG1;
        const ulong *pS2 = pG2;
        if (nM > 0) {
            BitGeneUtils::crossOver(m_vTmp1.data(), pG1, m_iGenomeSize, nM, m_apWELL[iT]);
            pS1 = m_vTmp1.data();
        }
        if (nF > 0) {
            BitGeneUtils::crossOver(m_vTmp2.data(), pG2, m_iGenomeSize, nF, m_apWELL[iT]);
            pS2 = m_vTmp2.data();
        }
        memcpy(pBaby, pS1 + i1*m_iNumBlocks, m_iNumBlocks*sizeof(ulong));
        memcpy(pBaby + m_iNumBlocks, pS2 + i2*m_iNumBlocks, m_iNumBlocks*sizeof(ulong));
        if (m_pGenetics->mutationRate() > 0) {
            int iNumMutations = m_pBDistPoisson->getN(m_apWELL[iT]->wrandd());
            if (iNumMutations > 0) {
                BitGeneUtils::mutateNucs(pBaby, 2*m_iGenomeSize, iNumMutations, m_apWELL[iT]);
            }
        }
        return 0;
    }

    void prioLevels(std::set<uint> &sPrios) {
        m_prio.getPrios(sPrios);
    }

    ulong countLive() {
        ulong n = 0;
        for (int c = 0; c < m_iNumCells; c++) n += m_aiNumAgentsPerCell[c];
        return n;
    }

    HarnessGenetics *m_pGenetics;
    HarnessMoveStats *m_pMoveStats = NULL;
    double *m_adK;
    double *m_adWeights;
    idtype m_iNextID;
    int m_iGenomeSize;
    int m_iNumBlocks;
    int m_iCrossMode;
    BinomialDist *m_pBDistPoisson = NULL;
    std::vector<ulong> m_vTmp1, m_vTmp2;
    std::vector<Action<RefAgent>*> m_vOwned;
    std::vector<double*> m_vTemp;
    std::vector<ActionSpec> m_vSpecs;
    std::vector<Action<RefAgent>*> m_vSpecActions;
    std::map<Action<RefAgent>*, uint32_t> m_mWindowBase, m_mWindowSize;
    std::vector<int64_t> m_vBirthLog;
    ulong m_iStepBirths = 0, m_iStepDeaths = 0, m_iStepMoves = 0;
};

/* ---------------------------------------------------------------------- */
static bool rd(FILE *f, void *p, size_t sz, size_t n) {
    return (n == 0) || (fread(p, sz, n, f) == n);
}
static void wr(FILE *f, const void *p, size_t sz, size_t n) {
    if (n > 0) fwrite(p, sz, n, f);
}

/* splitmix64, used to expand a seed into the 16-word WELL state */
static uint64_t splitmix64(uint64_t &x) {
    uint64_t z = (x += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

int main(int argc, char *argv[]) {
    if (argc < 3) {
        fprintf(stderr, "usage: %s <input.bin> <output.bin>\n", argv[0]);
        return 2;
    }
    FILE *fIn = fopen(argv[1], "rb");
    if (fIn == NULL) { fprintf(stderr, "cannot open %s\n", argv[1]); return 2; }
    char magic[8];
    uint32_t C, N, nSteps, iLayer;
    uint64_t seed;
    uint32_t nAct;
    bool ok = rd(fIn, magic, 1, 8) && (memcmp(magic, "QHGREF01", 8) == 0);
    ok = ok && rd(fIn, &C, 4, 1) && rd(fIn, &N, 4, 1) && rd(fIn, &nSteps, 4, 1) && rd(fIn, &iLayer, 4, 1);
    ok = ok && rd(fIn, &seed, 8, 1) && rd(fIn, &nAct, 4, 1);
    std::vector<ActionSpec> vSpecs(ok ? nAct : 0);
    for (uint32_t i = 0; ok && (i < nAct); i++) {
        ok = rd(fIn, &vSpecs[i].type, 4, 1) && rd(fIn, &vSpecs[i].prio, 4, 1) && rd(fIn, vSpecs[i].p, 8, 4);
    }
    uint32_t iGenomeSize = 0, iDumpEvery = 0;
    int32_t iCross = 0;
    double dMut = 0;
    ok = ok && rd(fIn, &iGenomeSize, 4, 1) && rd(fIn, &iCross, 4, 1) && rd(fIn, &dMut, 8, 1) && rd(fIn, &iDumpEvery, 4, 1);
    std::vector<int32_t> vNbr(ok ? (size_t)C*6 : 0);
    std::vector<uint8_t> vNN(ok ? C : 0);
    std::vector<double> vK(ok ? C : 0);
    ok = ok && rd(fIn, vNbr.data(), 4, vNbr.size()) && rd(fIn, vNN.data(), 1, C) && rd(fIn, vK.data(), 8, C);
    std::vector<int64_t> vID(ok ? N : 0);
    std::vector<int32_t> vCell(ok ? N : 0);
    std::vector<float> vBirth(ok ? N : 0), vAge(ok ? N : 0), vLB(ok ? N : 0);
    std::vector<uint8_t> vG(ok ? N : 0), vS(ok ? N : 0);
    ok = ok && rd(fIn, vID.data(), 8, N) && rd(fIn, vCell.data(), 4, N) && rd(fIn, vBirth.data(), 4, N)
            && rd(fIn, vAge.data(), 4, N) && rd(fIn, vLB.data(), 4, N) && rd(fIn, vG.data(), 1, N)
            && rd(fIn, vS.data(), 1, N);
    size_t nWords = (iGenomeSize > 0) ? (size_t)N * 2 * ((iGenomeSize + 63) / 64) : 0;
    std::vector<uint64_t> vGen(ok ? nWords : 0);
    ok = ok && rd(fIn, vGen.data(), 8, nWords);
    /* optional: u32 has_weights, f64 W[C*7] if 1; u32 n_k_changes,
     * n_k_changes x (u32 step, f64 K[C]) */
    uint32_t iHasW = 0, nKC = 0;
    std::vector<double> vW;
    std::vector<uint32_t> vKCStep;
    std::vector<double> vKC;
    if (ok && rd(fIn, &iHasW, 4, 1)) {
        if (iHasW == 1) {
            vW.resize((size_t)C*7);
            ok = rd(fIn, vW.data(), 8, vW.size());
        }
        ok = ok && rd(fIn, &nKC, 4, 1);
        vKCStep.resize(ok ? nKC : 0);
        vKC.resize(ok ? (size_t)nKC*C : 0);
        for (uint32_t k = 0; ok && (k < nKC); k++) {
            ok = rd(fIn, &vKCStep[k], 4, 1) && rd(fIn, vKC.data() + (size_t)k*C, 8, C);
        }
    }
    /* optional: u32 movestats_mode + 1 (0 none), f64 radius, f64 lon[C], f64 lat[C] */
    uint32_t iMSMode1 = 0;
    double dMSRadius = 1.0;
    std::vector<double> vLon, vLat;
    bool bMS = ok && rd(fIn, &iMSMode1, 4, 1);
    if (bMS && (iMSMode1 > 0)) {
        vLon.resize(C);
        vLat.resize(C);
        ok = rd(fIn, &dMSRadius, 8, 1) && rd(fIn, vLon.data(), 8, C) && rd(fIn, vLat.data(), 8, C);
    }
    /* optional: u32 n_kill_events, (u32 step, u8 flags[C])...: before that
     * step every agent in a flagged cell dies, as FlatExpPop::updateEvent
     * kills agents in water or ice after a geography event */
    uint32_t nKill = 0;
    std::vector<uint32_t> vKillStep;
    std::vector<uint8_t> vKill;
    bool bKill = bMS && ok && rd(fIn, &nKill, 4, 1);
    if (bKill) {
        vKillStep.resize(nKill);
        vKill.resize((size_t)nKill * C);
        for (uint32_t k = 0; ok && (k < nKill); k++) {
            ok = rd(fIn, &vKillStep[k], 4, 1) && rd(fIn, vKill.data() + (size_t)k * C, 1, C);
        }
    }
    /* optional: u32 n_mods, (u32 step, u32 name_len, char name[name_len],
     * f64 value)...: runtime edits through Prioritizer::modifyAttributes
     * before that step */
    uint32_t nMods = 0;
    std::vector<uint32_t> vModStep;
    std::vector<std::string> vModName;
    std::vector<double> vModValue;
    if (bKill && ok && rd(fIn, &nMods, 4, 1)) {
        for (uint32_t k = 0; ok && (k < nMods); k++) {
            uint32_t iStepM = 0, iLen = 0;
            double dV = 0;
            ok = rd(fIn, &iStepM, 4, 1) && rd(fIn, &iLen, 4, 1) && (iLen < 256);
            std::string sName(ok ? iLen : 0, ' ');
            ok = ok && rd(fIn, &sName[0], 1, iLen) && rd(fIn, &dV, 8, 1);
            vModStep.push_back(iStepM);
            vModName.push_back(sName);
            vModValue.push_back(dV);
        }
    }
    /* optional: u32 has_ice, u8 ice[C] if has_ice == 1: the Geography's
     * m_abIce, which WeightedMove reads (actions/WeightedMove.cpp:91) */
    uint32_t iHasIce = 0;
    std::vector<uint8_t> vIce;
    if (bKill && ok && rd(fIn, &iHasIce, 4, 1) && (iHasIce == 1)) {
        vIce.resize(C);
        ok = rd(fIn, vIce.data(), 1, C);
    }
    fclose(fIn);
    if (!ok) { fprintf(stderr, "malformed input %s\n", argv[1]); return 2; }

    g_seed = seed;
    /* grid: ids are the cell indices, connectivity 6 (SURF_EQSAHEDRON) */
    stringmap smSurf;
    smSurf[SURF_TYPE] = SURF_EQSAHEDRON;
    SCellGrid *pCG = new SCellGrid(0, C, smSurf);
    pCG->m_aCells = new SCell[C];
    for (uint32_t c = 0; c < C; c++) {
        pCG->m_aCells[c].m_iGlobalID = (gridtype)c;
        pCG->m_aCells[c].m_iNumNeighbors = vNN[c];
        for (int j = 0; j < 6; j++) pCG->m_aCells[c].m_aNeighbors[j] = vNbr[(size_t)c*6+j];
        pCG->m_mIDIndexes[c] = c;
    }

    /* MoveStats reads cell coordinates from the grid's Geography, WeightedMove
     * its ice flags; the Geography exists before the actions are made, as
     * WeightedMove keeps the pointer it finds at construction */
    Geography *pGeo = NULL;
    if ((iMSMode1 > 0) || !vIce.empty()) {
        pGeo = new Geography(pCG, C, 6, dMSRadius);
        for (uint32_t c = 0; c < C; c++) {
            pGeo->m_adLongitude[c] = (iMSMode1 > 0) ? vLon[c] : 0.0;
            pGeo->m_adLatitude[c] = (iMSMode1 > 0) ? vLat[c] : 0.0;
            pGeo->m_abIce[c] = vIce.empty() ? false : (vIce[c] != 0);
        }
        pCG->setGeography(pGeo);
    }

    int nThreads = omp_get_max_threads();
    IDGen **apIDG = new IDGen*[nThreads];
    for (int t = 0; t < nThreads; t++) apIDG[t] = new IDGen(0, t, nThreads);
    uint32_t aulState[16];
    uint64_t sm = seed;
    for (int j = 0; j < 16; j++) aulState[j] = (uint32_t)splitmix64(sm);
    uint aiSeeds[NUM_SEEDS] = {0};

    OraclePop *pPop = new OraclePop(pCG, (iLayer > 0) ? (int)iLayer : 65536, apIDG, aulState, aiSeeds);
    if (pPop->setup(vSpecs, vK.data(), (int)iGenomeSize, iCross, dMut, (iHasW == 1) ? vW.data() : NULL,
                    (int)iMSMode1 - 1) != 0) {
        fprintf(stderr, "population setup failed\n");
        return 3;
    }
    pPop->loadAgents(N, vID.data(), vCell.data(), vBirth.data(), vAge.data(), vLB.data(), vG.data(), vS.data(), vGen.data());
    pPop->preLoop();

    std::vector<uint64_t> vStats;
    std::vector<uint32_t> vDumpSteps;
    std::vector<uint32_t> vDumps;
    std::set<uint> sPrios;
    double t0 = omp_get_wtime();
    ulong iAgentSteps = 0;
    for (uint32_t s = 0; s < nSteps; s++) {
        g_curStep = (int)s;
        float fT = (float)s;
        iAgentSteps += pPop->countLive();
        for (uint32_t k = 0; k < nKC; k++) {
            if (vKCStep[k] == s) pPop->setK(vKC.data() + (size_t)k*C);
        }
        for (uint32_t k = 0; k < nKill; k++) {
            if (vKillStep[k] == s) pPop->killInCells(vKill.data() + (size_t)k*C);
        }
        for (uint32_t k = 0; k < nMods; k++) {
            if (vModStep[k] == s) pPop->modify(vModName[k], vModValue[k]);
        }
        /* PopLooper::doStep (core/PopLooper.cpp:166-200) */
        int iRes = pPop->initializeStep(fT);
        sPrios.clear();
        pPop->prioLevels(sPrios);
        for (std::set<uint>::const_iterator it = sPrios.begin(); it != sPrios.end(); ++it) {
            iRes += pPop->doActions(*it, fT);
        }
        iRes += pPop->finalizeStep();
        if (iRes != 0) {
            fprintf(stderr, "step %u returned %d\n", s, iRes);
        }
        vStats.push_back(pPop->countLive());
        vStats.push_back(pPop->m_iStepBirths);
        vStats.push_back(pPop->m_iStepDeaths);
        vStats.push_back(pPop->m_iStepMoves);
        if ((iDumpEvery > 0) && (((s + 1) % iDumpEvery) == 0)) {
            vDumpSteps.push_back(s);
            ulong *pN = pPop->getNumAgentsArray();
            for (uint32_t c = 0; c < C; c++) vDumps.push_back((uint32_t)pN[c]);
        }
    }
    double t1 = omp_get_wtime();

    /* live agents sorted by ID */
    std::vector<std::pair<int64_t,int> > vLive;
    int iFirst = pPop->getFirstAgentIndex();
    if (iFirst != LBController::NIL) {
        int iLast = pPop->getLastAgentIndex();
        for (int iA = iFirst; iA <= iLast; iA++) {
            if (pPop->m_aAgents[iA].m_iLifeState > 0) {
                vLive.push_back(std::make_pair((int64_t)pPop->m_aAgents[iA].m_ulID, iA));
            }
        }
    }
    std::sort(vLive.begin(), vLive.end());

    FILE *fOut = fopen(argv[2], "wb");
    if (fOut == NULL) { fprintf(stderr, "cannot open %s\n", argv[2]); return 2; }
    wr(fOut, "QHGOUT01", 1, 8);
    wr(fOut, &nSteps, 4, 1);
    wr(fOut, &C, 4, 1);
    wr(fOut, vStats.data(), 8, vStats.size());
    uint32_t nDumps = (uint32_t)vDumpSteps.size();
    wr(fOut, &nDumps, 4, 1);
    wr(fOut, vDumpSteps.data(), 4, nDumps);
    wr(fOut, vDumps.data(), 4, vDumps.size());
    uint64_t nLive = vLive.size();
    wr(fOut, &nLive, 8, 1);
    std::vector<int64_t> oID(nLive); std::vector<int32_t> oCell(nLive);
    std::vector<float> oB(nLive), oA(nLive), oL(nLive); std::vector<uint8_t> oG(nLive), oS(nLive);
    int nb = (iGenomeSize > 0) ? pPop->m_iNumBlocks : 0;
    std::vector<uint64_t> oGen((size_t)nLive * 2 * nb);
    for (size_t i = 0; i < nLive; i++) {
        RefAgent &a = pPop->m_aAgents[vLive[i].second];
        oID[i] = a.m_ulID; oCell[i] = a.m_iCellIndex; oB[i] = a.m_fBirthTime; oA[i] = a.m_fAge;
        oL[i] = a.m_fLastBirth; oG[i] = a.m_iGender; oS[i] = (uint8_t)a.m_iLifeState;
        if (nb > 0) memcpy(&oGen[i*2*nb], pPop->m_pGenetics->getGenome(vLive[i].second), 2*nb*sizeof(uint64_t));
    }
    wr(fOut, oID.data(), 8, nLive); wr(fOut, oCell.data(), 4, nLive); wr(fOut, oB.data(), 4, nLive);
    wr(fOut, oA.data(), 4, nLive); wr(fOut, oL.data(), 4, nLive); wr(fOut, oG.data(), 1, nLive);
    wr(fOut, oS.data(), 1, nLive); wr(fOut, oGen.data(), 8, oGen.size());
    uint64_t nBL = pPop->m_vBirthLog.size() / 3;
    wr(fOut, &nBL, 8, 1);
    for (int k = 0; k < 3; k++) {
        for (uint64_t i = 0; i < nBL; i++) wr(fOut, &pPop->m_vBirthLog[3*i+k], 8, 1);
    }
#ifdef QHG_PHILOX_TEST_BUILD
    uint64_t nErr = g_qhgDrawErrors;
#else
    uint64_t nErr = 0;
#endif
    wr(fOut, &nErr, 8, 1);
    double dSec = t1 - t0;
    wr(fOut, &dSec, 8, 1);
    uint64_t uAS = iAgentSteps;
    wr(fOut, &uAS, 8, 1);
    uint32_t uThr = (uint32_t)nThreads;
    wr(fOut, &uThr, 4, 1);
    /* MoveStats: u32 present, i32 hops[C], f64 dist[C], f64 time[C] */
    uint32_t uMS = (pPop->m_pMoveStats != NULL) ? 1 : 0;
    wr(fOut, &uMS, 4, 1);
    if (uMS) {
        wr(fOut, pPop->m_pMoveStats->hops(), 4, C);
        wr(fOut, pPop->m_pMoveStats->dist(), 8, C);
        wr(fOut, pPop->m_pMoveStats->time(), 8, C);
    }
    fclose(fOut);
    fprintf(stderr, "done: %u steps, %lu live, %.3f s, %.3g agent-steps/s, %d threads, draw errors %lu\n",
            nSteps, (unsigned long)nLive, dSec, dSec > 0 ? iAgentSteps / dSec : 0.0, nThreads, (unsigned long)nErr);
    return (nErr == 0) ? 0 : 4;
}
