/*
 * GpuSexualPop: the tutorial sexual population (GetOld, Fertility,
 * RandomPair, Verhulst, RandomMove; populations/tut_SexualPop.cpp:24-43) with
 * its step on the GPU (GpuPop.h).  Parameters are set by setParams with the
 * reference's attribute names (Fertility_min_age, Fertility_max_age,
 * Fertility_interbirth, Verhulst_b0, Verhulst_d0, Verhulst_theta, Verhulst_K,
 * RandomMove_prob), "name=value" pairs separated by ';'.
 */
#ifndef QHG_GPUSEXUALPOP_H
#define QHG_GPUSEXUALPOP_H

#include "GpuPop.h"

struct GpuSexualAgent : Agent {
    float m_fAge;
    float m_fLastBirth;
    int m_iMateIndex;
};

class GpuSexualPop : public GpuPop<GpuSexualAgent> {
public:
    GpuSexualPop(SCellGrid *pCG, PopFinder *pPopFinder, int iLayerSize, IDGen **apIDG, uint32_t *aulState,
                 uint *aiSeeds);
    virtual ~GpuSexualPop() {}

    virtual int setParams(const std::string sParams);
    virtual int preLoop();
    int addPopSpecificAgentData(int iAgentIndex, char **ppData);
    int makePopSpecificOffspring(int iAgent, int iMother, int iFather);

protected:
    double m_dFertMin, m_dFertMax, m_dInterbirth;
    double m_dB0, m_dD0, m_dTheta, m_dK;
    double m_dMoveProb;
};

#endif
