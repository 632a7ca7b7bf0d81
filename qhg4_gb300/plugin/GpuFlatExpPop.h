/*
 * GpuFlatExpPop: the FlatExpPop population (populations/FlatExpPop.cpp:32-91)
 * with its step on the GPU (GpuPop.h).
 *
 * Its environment evaluators stay on the host as the reference's own
 * objects: NPPCapacity turns the vegetation's NPP into capacities, two
 * SingleEvaluators (altitude, NPP) feed a MultiEvaluator that leaves
 * WeightedMove's cumulative weights.  They read their attributes from the
 * configuration under their own names, run in initializeStep, and their
 * weights go to the GPU run before the first step and after each
 * environment event (qhg_gpu_set_move_weights).  The agent actions --
 * Fertility, RandomPair, Verhulst, GetOld, OldAgeDeath, WeightedMove -- are
 * GpuParamActions: their attributes and priorities come from the same
 * configuration modules the reference's actions read.
 *
 * Genomes: the reference's Genetics object stays on the host for what it
 * does there -- its attributes, the initial genomes (createInitialGenomes in
 * preLoop, as FlatExpPop::preLoop calls it) and the genome buffer beside the
 * agents that QDF writing reads; crossover and mutation of the newborns run
 * on the GPU (setGpuGenetics), and preWrite brings the genomes back.
 *
 * Events: after a geography event the agents in water or ice cells die
 * before the next step (GpuPop::removeAgentsInCells), as in
 * FlatExpPop::updateEvent; every event is passed on to the evaluators
 * (notifyObservers) and marks the environment arrays for the next step.
 */
#ifndef QHG_GPUFLATEXPPOP_H
#define QHG_GPUFLATEXPPOP_H

#include "GpuPop.h"
#include "BitGeneUtils.h"
#include "Genetics.h"
#include "Geography.h"
#include "MultiEvaluator.h"
#include "NPPCapacity.h"
#include "SingleEvaluator.h"

struct GpuFlatExpAgent : Agent {
    float m_fAge;
    float m_fLastBirth;
    int m_iMateIndex;
    int m_iNumBabies;
};

// the reference's Genetics with the parameters it read readable
class GpuFlatExpGenetics : public Genetics<GpuFlatExpAgent, BitGeneUtils> {
public:
    GpuFlatExpGenetics(SPopulation<GpuFlatExpAgent> *pPop, SCellGrid *pCG, LBController *pAgentController,
                       std::vector<int> *pvDeadList, WELL512 **apWELL)
        : Genetics<GpuFlatExpAgent, BitGeneUtils>(pPop, pCG, "", pAgentController, pvDeadList, apWELL) {}
    int numCrossOvers() const { return m_iNumCrossOvers; }
    double mutationRate() const { return m_dMutationRate; }
    // newborns' genomes are made by the GPU run
    virtual int initialize(float fT) { return 0; }
    virtual int execute(int iA, float fT) { return 0; }
    virtual int finalize(float fT) { return 0; }
};

class GpuFlatExpPop : public GpuPop<GpuFlatExpAgent> {
public:
    GpuFlatExpPop(SCellGrid *pCG, PopFinder *pPopFinder, int iLayerSize, IDGen **apIDG, uint32_t *aulState,
                  uint *aiSeeds);
    virtual ~GpuFlatExpPop();

    virtual int prepareGpu();
    virtual int updateEvent(int iEventID, char *pData, float fT);
    virtual void flushEvents(float fT);
    int addPopSpecificAgentData(int iAgentIndex, char **ppData);
    int makePopSpecificOffspring(int iAgent, int iMother, int iFather);

protected:
    double *m_adCapacities;    // NPPCapacity's output, the NPP evaluator's input
    double *m_adEnvWeights;    // the MultiEvaluator's cumulative weights, cells x (connectivity + 1)
    NPPCapacity<GpuFlatExpAgent> *m_pNPPCap;
    MultiEvaluator<GpuFlatExpAgent> *m_pME;
    GpuFlatExpGenetics *m_pGenetics;
};

#endif
