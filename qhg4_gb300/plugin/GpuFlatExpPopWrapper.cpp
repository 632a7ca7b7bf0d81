// dynpops entry points of GpuFlatExpPop (the loader's ABI,
// dynpops/WrapperTemplate.cpp.tmp:14-30, populations/DynPopFactory.cpp:91-150)
#include <string>

#include "ArrayShare.h"
#include "IDGen.h"
#include "PopBase.h"
#include "PopFinder.h"
#include "SCellGrid.h"
#include "GpuFlatExpPop.h"

extern "C" {
const std::string getInfo() { return "GpuFlatExpPop"; }

PopBase *createPop(ArrayShare *pAS, SCellGrid *pCG, PopFinder *pPopFinder, int iLayerSize, IDGen **apIDG,
                   uint32_t *aulState, uint *aiSeeds) {
    ArrayShare::setInstance(pAS);
    // the loader calls createPop with six arguments (populations/DynPopFactory.cpp:18,150):
    // aiSeeds is not valid; SPopulation's constructor copies NUM_SEEDS values
    // from the pointer it gets (core/SPopulation.cpp:82), so it gets zeros
    static uint s_aiNoSeeds[NUM_SEEDS] = {0};
    (void)aiSeeds;
    return new GpuFlatExpPop(pCG, pPopFinder, iLayerSize, apIDG, aulState, s_aiNoSeeds);
}
}
