// Configuration check of GpuPop's GpuParamActions, without a GPU: a
// population with one parameter action of every QHG_ACT_* type gets its
// priorities through SPopulation::setPrioList and its attributes through
// Prioritizer::getActionAttributes, as QHG4 configures a population from its
// XML/QDF modules, and prints the action list the GPU run would be created
// with, one line per action: "type prio name p0 p1 p2 p3".  Then a module
// without one of its attributes must be refused ("missing <rc>"); equal
// configurations compare equal (Action::isEqual, "equal 1") until a runtime
// edit changes one ("edited <rc> <equal>").
//
// Built by `make -C qhg4_gb300/plugin param_check` against the reference tree
// and the reference's support objects (tests/test_plugin_build.py).
#include <cstdio>
#include <map>
#include <string>

#include "GpuSexualPop.cpp"

static uint s_aiSeeds[NUM_SEEDS] = {0};

class ParamCheckPop : public GpuPop<GpuSexualAgent> {
public:
    ParamCheckPop(SCellGrid *pCG, IDGen **apIDG, uint32_t *aulState)
        : GpuPop<GpuSexualAgent>(pCG, NULL, 1024, apIDG, aulState, s_aiSeeds) {
        for (int32_t t = QHG_ACT_GETOLD; t <= QHG_ACT_ATANDEATH; t++) addGpuParamAction(t);
    }

    int configure(const std::map<std::string, int> &mPrios, const modulemap &mModules) {
        m_mPrioInfo = mPrios;
        int iResult = setPrioList();
        if (iResult == 0) iResult = m_prio.getActionAttributes(mModules);
        return iResult;
    }

    bool sameActions(ParamCheckPop *pOther) {
        for (size_t k = 0; k < m_vParamActions.size(); k++) {
            if (!m_vParamActions[k]->isEqual(pOther->m_vParamActions[k], true)) return false;
        }
        return true;
    }

    int edit(const std::string &sName, double dValue) { return m_prio.modifyAttributes(sName, dValue); }

    void show() {
        collectParamActions();
        const std::vector<GpuAction> v = actionList();
        for (size_t i = 0; i < v.size(); i++) {
            const GpuAction &a = v[i];
            printf("%d %u %s %.17g %.17g %.17g %.17g\n", a.iType, a.iPrio, a.sName.c_str(), a.adP[0], a.adP[1],
                   a.adP[2], a.adP[3]);
        }
    }
};

static ModuleComplex *module(std::map<std::string, std::string> m) {
    ModuleComplex *p = new ModuleComplex();
    for (std::map<std::string, std::string>::const_iterator it = m.begin(); it != m.end(); ++it) {
        p->addParam(it->first, it->second);
    }
    return p;
}

int main() {
    // a ring of 4 cells
    stringmap smSurf;
    smSurf[SURF_TYPE] = SURF_EQSAHEDRON;
    const int C = 4;
    SCellGrid *pCG = new SCellGrid(0, C, smSurf);
    pCG->m_aCells = new SCell[C];
    for (int c = 0; c < C; c++) {
        pCG->m_aCells[c].m_iGlobalID = c;
        pCG->m_aCells[c].m_iNumNeighbors = 2;
        for (int j = 0; j < 6; j++) pCG->m_aCells[c].m_aNeighbors[j] = -1;
        pCG->m_aCells[c].m_aNeighbors[0] = (c + 1) % C;
        pCG->m_aCells[c].m_aNeighbors[1] = (c + C - 1) % C;
        pCG->m_mIDIndexes[c] = c;
    }
    int nThreads = omp_get_max_threads();
    IDGen **apIDG = new IDGen*[nThreads];
    for (int t = 0; t < nThreads; t++) apIDG[t] = new IDGen(0, t, nThreads);
    uint32_t aulState[16] = {7, 9};

    std::map<std::string, int> mPrios = {
        {"GetOld", 8}, {"Fertility", 2}, {"RandomPair", 3}, {"Verhulst", 6}, {"VerhulstVarK", 6},
        {"OldAgeDeath", 4}, {"RandomMove", 7}, {"WeightedMove", 7}, {"ATanDeath", 5}};
    modulemap mModules;
    mModules["Fertility"] = module({{"Fertility_min_age", "15"}, {"Fertility_max_age", "45.5"},
                                    {"Fertility_interbirth", "2"}});
    mModules["Verhulst"] = module({{"Verhulst_b0", "0.2"}, {"Verhulst_d0", "0.05"}, {"Verhulst_theta", "0.01"},
                                   {"Verhulst_K", "30"}});
    mModules["VerhulstVarK"] = module({{"Verhulst_b0", "0.25"}, {"Verhulst_d0", "0.04"}, {"Verhulst_theta", "0.02"}});
    mModules["OldAgeDeath"] = module({{"OAD_max_age", "64"}, {"OAD_uncertainty", "0.078125"}});
    mModules["RandomMove"] = module({{"RandomMove_prob", "0.1"}});
    mModules["WeightedMove"] = module({{"WeightedMove_prob", "0.2"}});
    mModules["ATanDeath"] = module({{"ATanDeath_max_age", "55"}, {"ATanDeath_range", "12"},
                                    {"ATanDeath_slope", "0.35"}});
    ParamCheckPop *pPop = new ParamCheckPop(pCG, apIDG, aulState);
    int iResult = pPop->configure(mPrios, mModules);
    if (iResult != 0) {
        printf("configure failed %d\n", iResult);
        return 1;
    }
    pPop->show();

    ParamCheckPop *pSame = new ParamCheckPop(pCG, apIDG, aulState);
    pSame->configure(mPrios, mModules);
    printf("equal %d\n", pPop->sameActions(pSame) ? 1 : 0);
    const int iEdit = pSame->edit("RandomMove_prob", 0.3);
    printf("edited %d %d\n", iEdit, pPop->sameActions(pSame) ? 1 : 0);

    // a module that lacks an attribute is refused
    ParamCheckPop *pPop2 = new ParamCheckPop(pCG, apIDG, aulState);
    delete mModules["RandomMove"];
    mModules["RandomMove"] = module({{"RandomMove_probability", "0.1"}});
    printf("missing %d\n", pPop2->configure(mPrios, mModules));
    return 0;
}
