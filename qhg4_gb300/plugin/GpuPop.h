/*
 * GpuPop<T>: a QHG4 population whose per-step update runs on the GPU
 * through libqhg_gpu.so (include/qhg_gpu.h), as a drop-in for the CPU
 * SPopulation<T> (core/SPopulation.h:86-107) under QHG4's PopLooper
 * (core/PopLooper.cpp:166-200), loaded like every population through the
 * dynpops createPop/getInfo ABI (dynpops/WrapperTemplate.cpp.tmp:14-30).
 *
 * Compiled against the QHG4 source tree (its core/, actions/, utils/ and io/
 * headers); see Makefile in this directory.
 *
 * What changes against SPopulation<T>:
 *   preLoop        after SPopulation's preLoop: creates the GPU run from the
 *                  action list given by addGpuAction / addGpuParamAction
 *                  (types and parameters in QHG_ACT_* slots), uploads the
 *                  cell grid (SCellGrid neighbours), the capacity array and
 *                  the live agents of the LayerBuf (with their genomes, when
 *                  setGpuGenetics names the genome buffer)
 *   initializeStep runs the initialize of the environment evaluators that
 *                  stay on the host (addHostEvaluator: the reference's own
 *                  NPPCapacity, SingleEvaluator, MultiEvaluator objects) and,
 *                  after an environment event, hands the arrays they fill
 *                  (setGpuEnvironment: K per cell, cumulative move weights)
 *                  to the GPU run; nothing else: the GPU step does pairing,
 *                  rates, every action's execute, births, deaths, moves and
 *                  counts
 *   doActions      nothing
 *   finalizeStep   one qhg_gpu_step; counts are read back when asked for
 *   updateNumAgentsPerCell, updateTotal
 *                  per-cell counts and total from the GPU
 *   preWrite, postLoop
 *                  copy the GPU table back into the LayerBuf first, so that
 *                  the reference's writers see the current agents
 *
 * Draws come from the keyed Philox stream of the GPU library (seed, step,
 * agent ID, action): a GPU population reproduces the reference's Philox
 * test build bit for bit and the stock WELL512 populations in distribution.
 * T must be the reference's Agent with m_fAge and m_fLastBirth.
 */
#ifndef QHG_GPUPOP_H
#define QHG_GPUPOP_H

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <set>
#include <string>
#include <vector>

#include "Action.h"
#include "ParamProvider2.h"
#include "QDFUtils.h"
#include "QDFUtilsT.h"
#include "SPopulation.h"
#include "Fertility.h"
#include "GetOld.h"
#include "OldAgeDeath.h"
#include "RandomMove.h"
#include "RandomPair.h"
#include "Verhulst.h"
#include "VerhulstVarK.h"
#include "WeightedMove.h"
#include "LBController.h"
#include "LayerArrBuf.h"
#include "SCellGrid.h"
#include "Geography.h"
#include "qhg_gpu.h"

// An action of a GPU population as the configuration sees it: it carries the
// reference action's name and attribute names, so that the population's
// Prioritizer hands it that action's module (Prioritizer::getActionAttributes,
// core/Prioritizer.cpp:440-462) and its priority (SPopulation::setPrioList);
// tryGetAttributes reads the attributes into the QHG_ACT_* parameter slots.
// Its execute is never called: the GPU step runs the action.
template<typename T>
class GpuParamAction : public Action<T> {
public:
    GpuParamAction(SPopulation<T> *pPop, SCellGrid *pCG, int32_t iType, const std::string &sName,
                   const std::vector<std::string> &vSlots)
        : Action<T>(pPop, pCG, sName, ""), m_iType(iType), m_vSlots(vSlots) {
        this->m_vNames.insert(this->m_vNames.end(), vSlots.begin(), vSlots.end());
        for (int k = 0; k < 4; k++) m_adP[k] = 0;
    }

    virtual int tryGetAttributes(const ModuleComplex *pMC) {
        const stringmap &mParams = pMC->getAttributes();
        int iResult = 0;
        for (size_t k = 0; (k < m_vSlots.size()) && (k < 4); k++) {
            stringmap::const_iterator it = mParams.find(m_vSlots[k]);
            if (it == mParams.end()) {
                iResult = -1;
                continue;
            }
            char *pEnd = NULL;
            m_adP[k] = strtod(it->second.c_str(), &pEnd);
            if (pEnd == it->second.c_str()) iResult = -1;
        }
        return iResult;
    }

    // QDF attributes under the reference action's names, so that a QDF file
    // of a GPU population and one of the reference's population read alike
    // (e.g. RandomMove::writeAttributesQDF, actions/RandomMove.cpp:130-137)
    virtual int writeAttributesQDF(hid_t hSpeciesGroup) {
        int iResult = 0;
        for (size_t k = 0; (k < m_vSlots.size()) && (k < 4); k++) {
            iResult += qdf_insertAttribute(hSpeciesGroup, m_vSlots[k], 1, &m_adP[k]);
        }
        return iResult;
    }

    virtual int extractAttributesQDF(hid_t hSpeciesGroup) {
        for (size_t k = 0; (k < m_vSlots.size()) && (k < 4); k++) {
            if (qdf_extractAttribute(hSpeciesGroup, m_vSlots[k], 1, &m_adP[k]) != 0) return -1;
        }
        return 0;
    }

    // the same action with the same parameters (Prioritizer::isEqual)
    virtual bool isEqual(Action<T> *pAction, bool bStrict) {
        GpuParamAction<T> *pA = dynamic_cast<GpuParamAction<T> *>(pAction);
        if ((pA == NULL) || (pA->m_iType != m_iType)) return false;
        for (int k = 0; k < 4; k++) {
            if (pA->m_adP[k] != m_adP[k]) return false;
        }
        return true;
    }

    // Runtime edits (Prioritizer::modifyAttributes, core/Prioritizer.cpp:420-434),
    // with the reference actions' effect: RandomMove and WeightedMove take a
    // new probability (actions/RandomMove.cpp:144-154,
    // actions/WeightedMove.cpp:153-163), which the GPU run gets before the
    // next step.  Verhulst / VerhulstVarK change their own fields but pass
    // the name to LinearBirth / LinearDeath, which know other names
    // (actions/Verhulst.cpp:235-255, actions/LinearBirth.cpp:235-248), so
    // their rates stay as they were and the call reports an error: the same
    // here.  The other actions have no runtime attributes.
    virtual int modifyAttributes(const std::string sAttrName, double dValue) {
        for (size_t k = 0; (k < m_vSlots.size()) && (k < 4); k++) {
            if (m_vSlots[k] != sAttrName) continue;
            if ((m_iType == QHG_ACT_RANDOMMOVE) || (m_iType == QHG_ACT_WEIGHTEDMOVE)) {
                m_adP[k] = dValue;
                m_bModified = true;
                return 0;
            }
            if ((m_iType == QHG_ACT_VERHULST) || (m_iType == QHG_ACT_VERHULSTVARK)) return -2;
        }
        return -1;
    }

    // the parameter action of a QHG_ACT_* type, with the reference's names
    // (actions/*.h ATTR_*), NULL for an unknown type
    static GpuParamAction<T> *create(SPopulation<T> *pPop, SCellGrid *pCG, int32_t iType) {
        switch (iType) {
        case QHG_ACT_GETOLD:
            return new GpuParamAction<T>(pPop, pCG, iType, ATTR_GETOLD_NAME, {});
        case QHG_ACT_FERTILITY:
            return new GpuParamAction<T>(pPop, pCG, iType, ATTR_FERTILITY_NAME,
                                         {ATTR_FERTILITY_MIN_AGE_NAME, ATTR_FERTILITY_MAX_AGE_NAME,
                                          ATTR_FERTILITY_INTERBIRTH_NAME});
        case QHG_ACT_RANDOMPAIR:
            return new GpuParamAction<T>(pPop, pCG, iType, ATTR_RANDPAIR_NAME, {});
        case QHG_ACT_VERHULST:
            return new GpuParamAction<T>(pPop, pCG, iType, ATTR_VERHULST_NAME,
                                         {ATTR_VERHULST_B0_NAME, ATTR_VERHULST_D0_NAME, ATTR_VERHULST_TURNOVER_NAME,
                                          ATTR_VERHULST_CAPACITY_NAME});
        case QHG_ACT_VERHULSTVARK:
            return new GpuParamAction<T>(pPop, pCG, iType, ATTR_VERHULSTVARK_NAME,
                                         {ATTR_VERHULSTVARK_B0_NAME, ATTR_VERHULSTVARK_D0_NAME,
                                          ATTR_VERHULSTVARK_TURNOVER_NAME});
        case QHG_ACT_OLDAGEDEATH:
            return new GpuParamAction<T>(pPop, pCG, iType, ATTR_OLDAGEDEATH_NAME,
                                         {ATTR_OLDAGEDEATH_MAXAGE_NAME, ATTR_OLDAGEDEATH_UNCERTAINTY_NAME});
        case QHG_ACT_RANDOMMOVE:
            return new GpuParamAction<T>(pPop, pCG, iType, ATTR_RANDOMMOVE_NAME, {ATTR_RANDOMMOVE_PROB_NAME});
        case QHG_ACT_WEIGHTEDMOVE:
            return new GpuParamAction<T>(pPop, pCG, iType, ATTR_WEIGHTEDMOVE_NAME, {ATTR_WEIGHTEDMOVE_PROB_NAME});
        case QHG_ACT_ATANDEATH:
            // actions/ATanDeath.h's names (that header's EPS would clash here)
            return new GpuParamAction<T>(pPop, pCG, iType, "ATanDeath",
                                         {"ATanDeath_max_age", "ATanDeath_range", "ATanDeath_slope"});
        default:
            return NULL;
        }
    }

    int32_t m_iType;
    std::vector<std::string> m_vSlots;
    double m_adP[4];
    bool m_bModified = false;   // a runtime edit the GPU run has not seen
};

template<typename T>
class GpuPop : public SPopulation<T> {
public:
    GpuPop(SCellGrid *pCG, PopFinder *pPopFinder, int iLayerSize, IDGen **apIDG, uint32_t *aulState,
           uint *aiSeeds)
        : SPopulation<T>(pCG, pPopFinder, iLayerSize, apIDG, aulState, aiSeeds),
          m_pRun(NULL), m_bStale(false), m_iDevice(0), m_adEnvK(NULL), m_adEnvW(NULL), m_bEnvDirty(true),
          m_iGenomeSize(0), m_iNumCrossover(0), m_dMutationRate(0), m_pGenome(NULL) {
        // the GPU run's seed from the population's generator state
        m_ulSeed = (aulState != NULL) ? ((uint64_t)aulState[0] | ((uint64_t)aulState[1] << 32)) : 0;
    }

    virtual ~GpuPop() {
        if (m_pRun != NULL) qhg_gpu_destroy(m_pRun);
        for (size_t i = 0; i < m_vParamActions.size(); i++) delete m_vParamActions[i];
    }

    // an action of the GPU step configured like the reference's: added to
    // the population's Prioritizer under the reference action's name, so that
    // its attributes and priority come from the configuration; preLoop hands
    // it to the GPU run
    int addGpuParamAction(int32_t iType) {
        GpuParamAction<T> *pA = GpuParamAction<T>::create(this, this->m_pCG, iType);
        if (pA == NULL) return -1;
        m_vParamActions.push_back(pA);
        this->m_prio.addAction(pA);
        return 0;
    }

    // one action: its QHG_ACT_* type, its priority and class name (the
    // execution order is SPopulation::setPrioList's: priority, then name)
    // and its parameter slots
    void addGpuAction(int32_t iType, uint iPrio, const std::string &sName, const double adP[4]) {
        GpuAction a;
        a.iType = iType;
        a.iPrio = iPrio;
        a.sName = sName;
        for (int k = 0; k < 4; k++) a.adP[k] = adP[k];
        m_vActions.push_back(a);
    }
    // capacity per cell (VerhulstVarK's K, WeightedMove's weights)
    void setGpuCapacity(const double *adK, int iNumCells) { m_vK.assign(adK, adK + iNumCells); }
    void setGpuDevice(int iDevice) { m_iDevice = iDevice; }
    // genetics of the run (Genetics_genome_size, Genetics_num_crossover or
    // QHG_CROSSOVER_POISSON1, Genetics_mutation_rate) and the genome buffer
    // the population keeps beside its agents (a LayerArrBuf of
    // 2 x ceil(size / 64) words per agent slot, strand 0 then strand 1, as
    // Genetics::m_aGenome, actions/Genetics.cpp:205-213, registered with the
    // agent controller): uploaded with the agents, written back by preWrite
    void setGpuGenetics(int iGenomeSize, int iNumCrossover, double dMutationRate, LayerArrBuf<ulong> *pGenome) {
        m_iGenomeSize = iGenomeSize;
        m_iNumCrossover = iNumCrossover;
        m_dMutationRate = dMutationRate;
        m_pGenome = pGenome;
    }
    // an environment evaluator kept on the host (not owned; also added to the
    // Prioritizer, which gives it its attributes and priority): its
    // initialize runs at each initializeStep and its finalize at each
    // finalizeStep, in priority order, as SPopulation's do for every action
    void addHostEvaluator(Action<T> *pA) {
        m_vHostEvals.push_back(pA);
        this->m_prio.addAction(pA);
    }
    // the arrays the host evaluators fill (not owned): K per cell (NULL:
    // none) and WeightedMove's cumulative weights, cells x 7 (NULL: the
    // weights follow K); handed to the GPU run before the first step and
    // after every environment event
    void setGpuEnvironment(const double *adK, const double *adCumW) {
        m_adEnvK = adK;
        m_adEnvW = adCumW;
        m_bEnvDirty = true;
    }

    virtual int preLoop() {
        int iResult = SPopulation<T>::preLoop();
        if (iResult == 0) iResult = prepareGpu();
        if (iResult == 0) collectParamActions();
        if (iResult == 0) iResult = startGpu();
        return iResult;
    }

    // between SPopulation's preLoop and the creation of the GPU run: what a
    // population's own preLoop does with its agents first (initial genomes)
    virtual int prepareGpu() { return 0; }

    virtual int initializeStep(float fTime) {
        if (m_pRun == NULL) return -1;
        int iResult = 0;
        if (paramsModified()) iResult = rebuildRun();
        for (size_t i = 0; i < m_vHostOrder.size(); i++) {
            iResult += m_vHostOrder[i]->initialize(fTime);
        }
        if ((iResult == 0) && m_bEnvDirty) {
            // the Geography's ice: WeightedMove registers no move into an ice
            // cell (actions/WeightedMove.cpp:91)
            const Geography *pGeo = this->m_pCG->m_pGeography;
            if ((pGeo != NULL) && (pGeo->m_abIce != NULL)) {
                std::vector<uint8_t> vIce((size_t)this->m_pCG->m_iNumCells);
                for (size_t c = 0; c < vIce.size(); c++) vIce[c] = pGeo->m_abIce[c] ? 1 : 0;
                if (qhg_gpu_set_ice(m_pRun, vIce.data()) != QHG_OK) iResult = -1;
            }
            if ((m_adEnvW != NULL) && (qhg_gpu_set_move_weights(m_pRun, m_adEnvW) != QHG_OK)) iResult = -1;
            if ((m_adEnvK != NULL) && (qhg_gpu_set_capacity(m_pRun, m_adEnvK) != QHG_OK)) iResult = -1;
            m_bEnvDirty = false;
        }
        return iResult;
    }

    // an environment event (climate, vegetation, geography) makes the host
    // evaluators recompute their arrays at the next initialize; they are
    // handed to the GPU run then
    virtual int updateEvent(int iEventID, char *pData, float fT) {
        m_bEnvDirty = true;
        return SPopulation<T>::updateEvent(iEventID, pData, fT);
    }
    virtual int doActions(uint iPrio, float fTime) { return 0; }

    virtual int finalizeStep() {
        if ((m_pRun == NULL) || (qhg_gpu_step(m_pRun, 1) != QHG_OK)) return -1;
        m_bStale = true;
        if (syncIDGens() != 0) return -1;
        // the host evaluators' finalize (an evaluator clears its update flag there)
        int iResult = 0;
        for (size_t i = 0; i < m_vHostOrder.size(); i++) {
            iResult += m_vHostOrder[i]->finalize(this->m_fCurTime);
        }
        return iResult;
    }

    virtual void updateNumAgentsPerCell() {
        if (m_pRun == NULL) {
            SPopulation<T>::updateNumAgentsPerCell();
            return;
        }
        pullCounts();
    }

    virtual void updateTotal() {
        if (m_pRun == NULL) {
            SPopulation<T>::updateTotal();
            return;
        }
        pullCounts();
    }

    virtual int preWrite(float fTime) {
        int iResult = copyBack();
        if (iResult == 0) iResult = SPopulation<T>::preWrite(fTime);
        return iResult;
    }

    virtual int postLoop() {
        int iResult = copyBack();
        if (m_pRun != NULL) {
            qhg_gpu_destroy(m_pRun);
            m_pRun = NULL;
        }
        if (iResult == 0) iResult = SPopulation<T>::postLoop();
        return iResult;
    }

    // the last error of the GPU library
    const char *gpuError() const { return qhg_gpu_last_error(); }

    // Every agent in a flagged cell dies now, before the next step -- what
    // FlatExpPop::updateEvent does after a geography event to agents in water
    // or ice (populations/FlatExpPop.cpp:187-214).  Such events are rare: the
    // run's table goes through the host (download, the flagged cells' agents
    // left out, upload at the run's step with its next ID kept).  The run's
    // occupation history and move statistics restart from that table.
    // Before the run exists the LayerBuf's agents are marked dead.
    int removeAgentsInCells(const uint8_t *aucRemove) {
        if (m_pRun == NULL) {
            const int iFirst = this->getFirstAgentIndex();
            if (iFirst != LBController::NIL) {
                for (int iA = iFirst; iA <= this->getLastAgentIndex(); iA++) {
                    T &a = this->m_aAgents[iA];
                    if ((a.m_iLifeState > 0) && aucRemove[a.m_iCellIndex]) a.m_iLifeState = 0;
                }
            }
            return 0;
        }
        int64_t n = 0, iNextID = 0;
        int32_t iStep = 0;
        if ((qhg_gpu_num_agents(m_pRun, &n) != QHG_OK) || (qhg_gpu_next_id(m_pRun, &iNextID) != QHG_OK) ||
            (qhg_gpu_current_step(m_pRun, &iStep) != QHG_OK)) {
            return -1;
        }
        const size_t nW = genomeWords();
        std::vector<int64_t> vID((size_t)n);
        std::vector<int32_t> vCell((size_t)n);
        std::vector<float> vBirth((size_t)n), vAge((size_t)n), vLast((size_t)n);
        std::vector<uint8_t> vGender((size_t)n), vState((size_t)n);
        std::vector<uint64_t> vGenome((size_t)n * nW);
        qhg_agents_soa s = {vID.data(), vCell.data(), vBirth.data(), vAge.data(), vLast.data(),
                            vGender.data(), vState.data(), (nW > 0) ? vGenome.data() : NULL};
        int64_t got = 0;
        if (qhg_gpu_download(m_pRun, &s, n, &got) != QHG_OK) return -1;
        int64_t k = 0;
        for (int64_t i = 0; i < got; i++) {
            if (aucRemove[vCell[(size_t)i]]) continue;
            vID[(size_t)k] = vID[(size_t)i];
            vCell[(size_t)k] = vCell[(size_t)i];
            vBirth[(size_t)k] = vBirth[(size_t)i];
            vAge[(size_t)k] = vAge[(size_t)i];
            vLast[(size_t)k] = vLast[(size_t)i];
            vGender[(size_t)k] = vGender[(size_t)i];
            vState[(size_t)k] = vState[(size_t)i];
            if (nW > 0) memmove(&vGenome[(size_t)k * nW], &vGenome[(size_t)i * nW], nW * sizeof(uint64_t));
            k++;
        }
        if ((qhg_gpu_upload_agents(m_pRun, &s, k, iStep) != QHG_OK) ||
            (qhg_gpu_set_next_id(m_pRun, iNextID) != QHG_OK)) {
            return -1;
        }
        m_bStale = true;
        pullCounts();
        return 0;
    }

protected:
    struct GpuAction {
        int32_t iType;
        uint iPrio;
        std::string sName;
        double adP[4];
    };

    // the parameter actions, in the Prioritizer's levels, into the action
    // list; the host evaluators in the same order
    void collectParamActions() {
        m_vHostOrder.clear();
        m_vParamGpu.clear();
        std::set<uint> sPrios;
        this->m_prio.getPrios(sPrios);
        for (std::set<uint>::const_iterator it = sPrios.begin(); it != sPrios.end(); ++it) {
            for (uint j = 0; j < this->m_prio.getNumActionsForPrio(*it); j++) {
                Action<T> *pA = this->m_prio.getAction(*it, j);
                for (size_t k = 0; k < m_vParamActions.size(); k++) {
                    if (m_vParamActions[k] == pA) {
                        GpuAction a;
                        a.iType = m_vParamActions[k]->m_iType;
                        a.iPrio = *it;
                        a.sName = pA->getActionName();
                        for (int q = 0; q < 4; q++) a.adP[q] = m_vParamActions[k]->m_adP[q];
                        m_vParamGpu.push_back(a);
                        m_vParamActions[k]->m_bModified = false;
                    }
                }
                if (std::find(m_vHostEvals.begin(), m_vHostEvals.end(), pA) != m_vHostEvals.end()) {
                    m_vHostOrder.push_back(pA);
                }
            }
        }
    }

    // the run's action list: the explicit actions and the parameter
    // actions, in execution order (priority, then name)
    std::vector<GpuAction> actionList() const {
        std::vector<GpuAction> v(m_vActions);
        v.insert(v.end(), m_vParamGpu.begin(), m_vParamGpu.end());
        std::stable_sort(v.begin(), v.end(), [](const GpuAction &a, const GpuAction &b) {
            return (a.iPrio != b.iPrio) ? (a.iPrio < b.iPrio) : (a.sName < b.sName);
        });
        return v;
    }

    bool paramsModified() const {
        for (size_t k = 0; k < m_vParamActions.size(); k++) {
            if (m_vParamActions[k]->m_bModified) return true;
        }
        return false;
    }

    // a new run with the edited parameters, holding the current one's table
    // (with genomes) at its step and with its next ID; the environment
    // arrays are handed over again at once
    int rebuildRun() {
        int64_t n = 0, iNextID = 0;
        int32_t iStep = 0;
        if ((qhg_gpu_num_agents(m_pRun, &n) != QHG_OK) || (qhg_gpu_next_id(m_pRun, &iNextID) != QHG_OK) ||
            (qhg_gpu_current_step(m_pRun, &iStep) != QHG_OK)) {
            return -1;
        }
        const size_t nW = genomeWords();
        std::vector<int64_t> vID((size_t)n);
        std::vector<int32_t> vCell((size_t)n);
        std::vector<float> vBirth((size_t)n), vAge((size_t)n), vLast((size_t)n);
        std::vector<uint8_t> vGender((size_t)n), vState((size_t)n);
        std::vector<uint64_t> vGenome((size_t)n * nW);
        qhg_agents_soa s = {vID.data(), vCell.data(), vBirth.data(), vAge.data(), vLast.data(),
                            vGender.data(), vState.data(), (nW > 0) ? vGenome.data() : NULL};
        int64_t got = 0;
        if (qhg_gpu_download(m_pRun, &s, n, &got) != QHG_OK) return -1;
        qhg_gpu_destroy(m_pRun);
        m_pRun = NULL;
        collectParamActions();
        if (createRun() != 0) return -1;
        if ((qhg_gpu_upload_agents(m_pRun, &s, got, iStep) != QHG_OK) ||
            (qhg_gpu_set_next_id(m_pRun, iNextID) != QHG_OK)) {
            return -1;
        }
        m_bEnvDirty = true;
        return 0;
    }

    // the GPU run with the action list, genetics and cell grid
    int createRun() {
        std::vector<GpuAction> v = actionList();
        if (v.size() > QHG_MAX_ACTIONS) return -1;
        qhg_run_desc d;
        memset(&d, 0, sizeof(d));
        d.seed = m_ulSeed;
        d.n_actions = (int32_t)v.size();
        for (size_t i = 0; i < v.size(); i++) {
            d.action_type[i] = v[i].iType;
            for (int k = 0; k < 4; k++) d.action_param[i][k] = v[i].adP[k];
        }
        d.device = m_iDevice;
        if (m_pGenome != NULL) {
            d.genome_size = m_iGenomeSize;
            d.num_crossover = m_iNumCrossover;
            d.mutation_rate = m_dMutationRate;
        }
        if (qhg_gpu_create(&d, &m_pRun) != QHG_OK) return -1;
        // grid: neighbours of each cell, -1 padded to 6
        const int C = (int)this->m_pCG->m_iNumCells;
        std::vector<int32_t> vNbr((size_t)C * 6, -1);
        std::vector<uint8_t> vN((size_t)C, 0);
        for (int c = 0; c < C; c++) {
            const SCell &cell = this->m_pCG->m_aCells[c];
            const int n = std::min<int>(cell.m_iNumNeighbors, 6);
            vN[c] = (uint8_t)n;
            for (int j = 0; j < n; j++) vNbr[(size_t)c * 6 + j] = (int32_t)cell.m_aNeighbors[j];
        }
        if (m_vK.size() != (size_t)C) m_vK.assign((size_t)C, 0.0);
        if (qhg_gpu_upload_grid(m_pRun, vNbr.data(), vN.data(), m_vK.data(), C) != QHG_OK) return -1;
        return 0;
    }

    int startGpu() {
        if (createRun() != 0) return -1;
        // live agents of the LayerBuf
        std::vector<int64_t> vID;
        std::vector<int32_t> vCell;
        std::vector<float> vBirth, vAge, vLast;
        std::vector<uint8_t> vGender, vState;
        std::vector<uint64_t> vGenome;
        const size_t nW = genomeWords();
        const int iFirst = this->getFirstAgentIndex();
        if (iFirst != LBController::NIL) {
            const int iLast = this->getLastAgentIndex();
            for (int iA = iFirst; iA <= iLast; iA++) {
                const T &a = this->m_aAgents[iA];
                if (a.m_iLifeState <= 0) continue;
                if (nW > 0) {
                    const ulong *g = &(*m_pGenome)[(uint)iA];
                    vGenome.insert(vGenome.end(), g, g + nW);
                }
                vID.push_back((int64_t)a.m_ulID);
                vCell.push_back((int32_t)a.m_iCellIndex);
                vBirth.push_back(a.m_fBirthTime);
                vAge.push_back(a.m_fAge);
                vLast.push_back(a.m_fLastBirth);
                vGender.push_back((uint8_t)a.m_iGender);
                vState.push_back((uint8_t)a.m_iLifeState);
            }
        }
        qhg_agents_soa s = {vID.data(), vCell.data(), vBirth.data(), vAge.data(), vLast.data(),
                            vGender.data(), vState.data(), (nW > 0) ? vGenome.data() : NULL};
        if (qhg_gpu_upload_agents(m_pRun, &s, (int64_t)vID.size(), 0) != QHG_OK) return -1;
        if (claimIDs() != 0) return -1;
        m_bStale = false;
        return 0;
    }

    // The ID generators are the application's, shared by all populations
    // (app/SimParams.cpp:138-141): the run's newborns took IDs from its own
    // counter, so every generator is moved past it (never back), and QHG4's
    // dumps record it (IDGen::getCur, core/IDGen.h).
    int syncIDGens() {
        int64_t iNextID = 0;
        if (qhg_gpu_next_id(m_pRun, &iNextID) != QHG_OK) return -1;
        for (int t = 0; t < this->m_iNumThreads; t++) {
            IDGen *pG = this->m_apIDGen[t];
            const idtype iCur = pG->getCur();
            pG->setBase((idtype)iNextID);
            if (pG->getCur() < iCur) pG->setCur(iCur);
        }
        return 0;
    }

    // the run's first ID for newborns: above every ID in the table (the
    // upload's own choice) and every ID the generators have handed out
    int claimIDs() {
        int64_t iNextID = 0;
        if (qhg_gpu_next_id(m_pRun, &iNextID) != QHG_OK) return -1;
        for (int t = 0; t < this->m_iNumThreads; t++) {
            const int64_t iUsed = (int64_t)this->m_apIDGen[t]->getCur() + 1;
            if (iUsed > iNextID) iNextID = iUsed;
        }
        return (qhg_gpu_set_next_id(m_pRun, iNextID) == QHG_OK) ? 0 : -1;
    }

    // genome words per agent (0 without genetics)
    size_t genomeWords() const {
        return ((m_pGenome != NULL) && (m_iGenomeSize > 0)) ? 2 * (size_t)((m_iGenomeSize + 63) / 64) : 0;
    }

    void pullCounts() {
        const int C = (int)this->m_pCG->m_iNumCells;
        std::vector<uint32_t> v((size_t)C);
        if (qhg_gpu_counts(m_pRun, v.data()) != QHG_OK) return;
        ulong iTotal = 0;
        for (int c = 0; c < C; c++) {
            this->m_aiNumAgentsPerCell[c] = v[c];
            iTotal += v[c];
        }
        this->m_iTotal = iTotal;
    }

    // the GPU table into the LayerBuf (all slots rewritten)
    int copyBack() {
        if ((m_pRun == NULL) || !m_bStale) return 0;
        int64_t n = 0;
        if (qhg_gpu_num_agents(m_pRun, &n) != QHG_OK) return -1;
        std::vector<int64_t> vID((size_t)n);
        std::vector<int32_t> vCell((size_t)n);
        std::vector<float> vBirth((size_t)n), vAge((size_t)n), vLast((size_t)n);
        std::vector<uint8_t> vGender((size_t)n), vState((size_t)n);
        const size_t nW = genomeWords();
        std::vector<uint64_t> vGenome((size_t)n * nW);
        qhg_agents_soa s = {vID.data(), vCell.data(), vBirth.data(), vAge.data(), vLast.data(),
                            vGender.data(), vState.data(), (nW > 0) ? vGenome.data() : NULL};
        int64_t got = 0;
        if (qhg_gpu_download(m_pRun, &s, n, &got) != QHG_OK) return -1;
        this->m_pAgentController->clear();
        if (got > 0) {
            const int iStart = (int)this->m_pAgentController->reserveSpace2((uint)got);
            for (int64_t i = 0; i < got; i++) {
                T &a = this->m_aAgents[iStart + (int)i];
                a.m_iLifeState = vState[(size_t)i];
                a.m_iCellIndex = vCell[(size_t)i];
                a.m_ulID = (idtype)vID[(size_t)i];
                a.m_ulCellID = this->m_pCG->m_aCells[vCell[(size_t)i]].m_iGlobalID;
                a.m_fBirthTime = vBirth[(size_t)i];
                a.m_iGender = vGender[(size_t)i];
                a.m_fAge = vAge[(size_t)i];
                a.m_fLastBirth = vLast[(size_t)i];
                if (nW > 0) {
                    memcpy(&(*m_pGenome)[(uint)(iStart + (int)i)], vGenome.data() + (size_t)i * nW,
                           nW * sizeof(uint64_t));
                }
            }
        }
        pullCounts();
        m_bStale = false;
        return 0;
    }

    qhg_run *m_pRun;
    bool m_bStale;
    int m_iDevice;
    uint64_t m_ulSeed;
    std::vector<GpuAction> m_vActions;
    std::vector<GpuAction> m_vParamGpu;   // the parameter actions' entries (collectParamActions)
    std::vector<double> m_vK;
    std::vector<Action<T> *> m_vHostEvals;
    std::vector<GpuParamAction<T> *> m_vParamActions;
    std::vector<Action<T> *> m_vHostOrder;   // the host evaluators in priority order
    const double *m_adEnvK;
    const double *m_adEnvW;
    bool m_bEnvDirty;
    int m_iGenomeSize;
    int m_iNumCrossover;
    double m_dMutationRate;
    LayerArrBuf<ulong> *m_pGenome;
};

#endif
