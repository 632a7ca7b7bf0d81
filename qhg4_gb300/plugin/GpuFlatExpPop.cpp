// the template code of the population and action classes, as the
// reference's populations include it (populations/FlatExpPop.cpp:1-25)
#include "EventConsts.h"
#include "SPopulation.cpp"
#include "LayerBuf.cpp"
#include "Prioritizer.cpp"
#include "Action.cpp"
#include "SingleEvaluator.cpp"
#include "MultiEvaluator.cpp"
#include "NPPCapacity.cpp"
#include "LayerArrBuf.cpp"
#include "Genetics.cpp"
#include "GenomeCreator.cpp"

#include <cstring>

#include "GpuFlatExpPop.h"

GpuFlatExpPop::GpuFlatExpPop(SCellGrid *pCG, PopFinder *pPopFinder, int iLayerSize, IDGen **apIDG,
                             uint32_t *aulState, uint *aiSeeds)
    : GpuPop<GpuFlatExpAgent>(pCG, pPopFinder, iLayerSize, apIDG, aulState, aiSeeds),
      m_adCapacities(NULL), m_adEnvWeights(NULL), m_pNPPCap(NULL), m_pME(NULL), m_pGenetics(NULL) {
    m_sSpeciesName = "GpuFlatExp";
    m_sClassName = "GpuFlatExpPop";
    const size_t C = (size_t)m_pCG->m_iNumCells;
    const size_t nW = C * (size_t)(m_pCG->m_iConnectivity + 1);
    m_adCapacities = new double[C];
    memset(m_adCapacities, 0, C * sizeof(double));
    m_adEnvWeights = new double[nW];
    memset(m_adEnvWeights, 0, nW * sizeof(double));

    // capacities from the vegetation's NPP (one value per cell)
    m_pNPPCap = new NPPCapacity<GpuFlatExpAgent>(this, m_pCG, "", m_apWELL, m_adCapacities, 1);
    // move weights: altitude and NPP preferences, added and cumulated by the
    // MultiEvaluator (which owns the two SingleEvaluators)
    MultiEvaluator<GpuFlatExpAgent>::evaluatorinfos vEvals;
    vEvals.push_back(std::make_pair(std::string("Multi_weight_alt"),
        (Evaluator<GpuFlatExpAgent> *)new SingleEvaluator<GpuFlatExpAgent>(
            this, m_pCG, "Alt", NULL, (m_pCG->m_pGeography != NULL) ? m_pCG->m_pGeography->m_adAltitude : NULL,
            "AltCapPref", true, EVENT_ID_GEO)));
    vEvals.push_back(std::make_pair(std::string("Multi_weight_npp"),
        (Evaluator<GpuFlatExpAgent> *)new SingleEvaluator<GpuFlatExpAgent>(
            this, m_pCG, "NPP", NULL, m_adCapacities, "NPPPref", true, EVENT_ID_VEG)));
    m_pME = new MultiEvaluator<GpuFlatExpAgent>(this, m_pCG, "Alt+NPP", m_adEnvWeights, vEvals,
                                                MultiEvalModes::MODE_ADD_SIMPLE, true);
    addHostEvaluator(m_pME);
    addHostEvaluator(m_pNPPCap);

    // the agent actions of the GPU step (Verhulst with its constant K)
    addGpuParamAction(QHG_ACT_WEIGHTEDMOVE);
    addGpuParamAction(QHG_ACT_VERHULST);
    addGpuParamAction(QHG_ACT_RANDOMPAIR);
    addGpuParamAction(QHG_ACT_GETOLD);
    addGpuParamAction(QHG_ACT_OLDAGEDEATH);
    addGpuParamAction(QHG_ACT_FERTILITY);

    // the genomes: the reference's Genetics for attributes, initial genomes
    // and the buffer beside the agents (its own step work is the GPU's)
    m_pGenetics = new GpuFlatExpGenetics(this, m_pCG, m_pAgentController, &m_vMergedDeadList, m_apWELL);
    m_prio.addAction(m_pGenetics);

    // the GPU run takes the weights as cells x 7 (connectivity 6)
    if (m_pCG->m_iConnectivity == 6) setGpuEnvironment(NULL, m_adEnvWeights);
}

GpuFlatExpPop::~GpuFlatExpPop() {
    delete m_pGenetics;
    delete m_pME;
    delete m_pNPPCap;
    delete[] m_adEnvWeights;
    delete[] m_adCapacities;
}

// after SPopulation's preLoop, as FlatExpPop::preLoop does: the initial
// genomes; the GPU run then gets the genetics the Genetics object read from
// the configuration and its genome buffer
int GpuFlatExpPop::prepareGpu() {
    int iResult = 0;
    if (m_pGenetics->getGenomeSize() > 0) {
        iResult = m_pGenetics->createInitialGenomes(getNumAgentsEffective());
        setGpuGenetics(m_pGenetics->getGenomeSize(), m_pGenetics->numCrossOvers(), m_pGenetics->mutationRate(),
                       m_pGenetics->getGenome());
    }
    return iResult;
}

// FlatExpPop::updateEvent (populations/FlatExpPop.cpp:187-219): a geography
// event drowns the agents in water or ice; every event goes on to the
// evaluators and marks the environment for the next step
int GpuFlatExpPop::updateEvent(int iEventID, char *pData, float fT) {
    int iResult = 0;
    Geography *pGeo = m_pCG->m_pGeography;
    if ((iEventID == EVENT_ID_GEO) && (pGeo != NULL)) {
        const size_t C = (size_t)m_pCG->m_iNumCells;
        std::vector<uint8_t> vRemove(C, 0);
        for (size_t c = 0; c < C; c++) {
            vRemove[c] = ((pGeo->m_adAltitude[c] < 0) || (pGeo->m_abIce[c] > 0)) ? 1 : 0;
        }
        iResult = removeAgentsInCells(vRemove.data());
    }
    if (iResult == 0) iResult = GpuPop<GpuFlatExpAgent>::updateEvent(iEventID, pData, fT);
    notifyObservers(iEventID, pData);
    return iResult;
}

// FlatExpPop::flushEvents
void GpuFlatExpPop::flushEvents(float fT) {
    notifyObservers(EVENT_ID_FLUSH, NULL);
}

// age and last birth time follow the basic agent data in the species' agent lines
int GpuFlatExpPop::addPopSpecificAgentData(int iAgentIndex, char **ppData) {
    int iResult = addAgentDataSingle(ppData, &m_aAgents[iAgentIndex].m_fAge);
    if (iResult == 0) iResult = addAgentDataSingle(ppData, &m_aAgents[iAgentIndex].m_fLastBirth);
    return iResult;
}

int GpuFlatExpPop::makePopSpecificOffspring(int iAgent, int iMother, int iFather) {
    m_aAgents[iAgent].m_fAge = 0.0f;
    m_aAgents[iAgent].m_fLastBirth = 0.0f;
    m_aAgents[iAgent].m_iMateIndex = -3;
    m_aAgents[iAgent].m_iNumBabies = 0;
    return 0;
}
