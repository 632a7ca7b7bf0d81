// the template code of the population classes, as the reference's own
// populations include it (e.g. populations/VirusHostPop.cpp:5-8)
#include "SPopulation.cpp"
#include "LayerBuf.cpp"
#include "Prioritizer.cpp"
#include "Action.cpp"

#include <cstdlib>
#include <sstream>

#include "GpuSexualPop.h"

GpuSexualPop::GpuSexualPop(SCellGrid *pCG, PopFinder *pPopFinder, int iLayerSize, IDGen **apIDG,
                           uint32_t *aulState, uint *aiSeeds)
    : GpuPop<GpuSexualAgent>(pCG, pPopFinder, iLayerSize, apIDG, aulState, aiSeeds),
      m_dFertMin(15), m_dFertMax(45), m_dInterbirth(2),
      m_dB0(0.2), m_dD0(0.05), m_dTheta(0.01), m_dK(30), m_dMoveProb(0.1) {
    m_sSpeciesName = "GpuSexual";
    m_sClassName = "GpuSexualPop";
}

// "name=value;name=value" with the reference's attribute names
int GpuSexualPop::setParams(const std::string sParams) {
    std::stringstream ss(sParams);
    std::string item;
    int iResult = 0;
    while (std::getline(ss, item, ';')) {
        const size_t eq = item.find('=');
        if (eq == std::string::npos) continue;
        const std::string k = item.substr(0, eq);
        const double v = atof(item.substr(eq + 1).c_str());
        if (k == "Fertility_min_age") m_dFertMin = v;
        else if (k == "Fertility_max_age") m_dFertMax = v;
        else if (k == "Fertility_interbirth") m_dInterbirth = v;
        else if (k == "Verhulst_b0") m_dB0 = v;
        else if (k == "Verhulst_d0") m_dD0 = v;
        else if (k == "Verhulst_theta") m_dTheta = v;
        else if (k == "Verhulst_K") m_dK = v;
        else if (k == "RandomMove_prob") m_dMoveProb = v;
        else iResult = -1;
    }
    return iResult;
}

// the tutorial population's priorities (tutorial_data/xmldat/tut_Sexual.xml):
// Fertility 2, RandomPair 3, Verhulst 6, RandomMove 7, GetOld 8
int GpuSexualPop::preLoop() {
    const double fert[4] = {m_dFertMin, m_dFertMax, m_dInterbirth, 0};
    const double none[4] = {0, 0, 0, 0};
    const double verh[4] = {m_dB0, m_dD0, m_dTheta, m_dK};
    const double move[4] = {m_dMoveProb, 0, 0, 0};
    m_vActions.clear();
    addGpuAction(QHG_ACT_FERTILITY, 2, "Fertility", fert);
    addGpuAction(QHG_ACT_RANDOMPAIR, 3, "RandomPair", none);
    addGpuAction(QHG_ACT_VERHULST, 6, "Verhulst", verh);
    addGpuAction(QHG_ACT_RANDOMMOVE, 7, "RandomMove", move);
    addGpuAction(QHG_ACT_GETOLD, 8, "GetOld", none);
    return GpuPop<GpuSexualAgent>::preLoop();
}

// age and last birth time follow the basic agent data in the species' agent lines
int GpuSexualPop::addPopSpecificAgentData(int iAgentIndex, char **ppData) {
    int iResult = addAgentDataSingle(ppData, &m_aAgents[iAgentIndex].m_fAge);
    if (iResult == 0) iResult = addAgentDataSingle(ppData, &m_aAgents[iAgentIndex].m_fLastBirth);
    return iResult;
}

int GpuSexualPop::makePopSpecificOffspring(int iAgent, int iMother, int iFather) {
    m_aAgents[iAgent].m_fAge = 0.0f;
    m_aAgents[iAgent].m_fLastBirth = 0.0f;
    m_aAgents[iAgent].m_iMateIndex = -3;
    return 0;
}
