/*
 * TEST INFRASTRUCTURE ONLY.  Runs the population plugin's GpuSexualPop the
 * way QHG4 runs a population: agents in its LayerBuf, SPopulation::preLoop,
 * then per step initializeStep / doActions per priority / finalizeStep
 * (PopLooper::doStep, core/PopLooper.cpp:166-200), and preWrite, which
 * copies the run's table back into the LayerBuf.  Linked against the
 * oracle-backed stand-in for libqhg_gpu.so (qhg_gpu_fake.c), so it runs
 * without a GPU; tests/test_plugin_host.py compares what it writes with the
 * reference's own tut_Sexual actions (the Philox test build).
 *
 *   plugin_drive <input> <output> [write_every] [param]
 * write_every > 0: preWrite every that many steps as well (QHG4 writes a
 * snapshot that way), the LayerBuf rewritten while the run goes on.
 * "param": the population's actions are the input's action list as
 * GpuParamActions, configured the way QHG4 configures a population --
 * priorities through SPopulation::setPrioList, attributes through
 * Prioritizer::getActionAttributes from one module per action -- with K per
 * cell from the input (VerhulstVarK, WeightedMove's weights).  The input's
 * optional environment -- given move weights, K changes at given steps --
 * is handed over as GpuPop's environment arrays: a K change rewrites the
 * array and raises an environment event before that step, as QHG4's event
 * manager does.  Kill events remove every agent of the flagged cells before
 * their step (GpuPop::removeAgentsInCells, a geography event's drowning);
 * runtime edits go through the Prioritizer's modifyAttributes before theirs.
 * input: the oracle harness's input format (oracle/refsim_io.py) with the
 * tutorial action set (and genomes, kept in a LayerArrBuf registered with the
 * agent controller as Genetics keeps them); output: u64 n, i64 id[n],
 * i32 cell[n], f32 birth[n], f32 age[n], f32 lastb[n], u8 gender[n],
 * u8 state[n], u32 C, u32 counts[C], u32 words, u64 genome[n * words],
 * i64 the smallest next ID of the population's ID generators.
 */
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "EventConsts.h"
#include "GpuSexualPop.cpp"
#include "LayerArrBuf.cpp"

class DrivePop : public GpuSexualPop {
public:
    DrivePop(SCellGrid *pCG, IDGen **apIDG, uint32_t *aulState, uint *aiSeeds)
        : GpuSexualPop(pCG, NULL, 65536, apIDG, aulState, aiSeeds) {}

    void prios(std::set<uint> &sPrios) { getPrios(sPrios); }

    // a runtime edit, as QHG4 applies one (Prioritizer::modifyAttributes)
    int modify(const std::string &sName, double dValue) { return m_prio.modifyAttributes(sName, dValue); }

    // the input's actions as parameter actions, configured from modules
    int configureActions(const std::vector<uint32_t> &vType, const std::vector<uint32_t> &vPrio,
                         const std::vector<double> &vP, const double *adK) {
        m_bParamMode = true;
        modulemap mModules;
        for (size_t i = 0; i < vType.size(); i++) {
            if (addGpuParamAction((int32_t)vType[i]) != 0) return -1;
            GpuParamAction<GpuSexualAgent> *pA = m_vParamActions.back();
            m_mPrioInfo[pA->getActionName()] = (int)vPrio[i];
            ModuleComplex *pMC = new ModuleComplex();
            char buf[64];
            for (size_t k = 0; k < pA->m_vSlots.size(); k++) {
                snprintf(buf, sizeof(buf), "%.17g", vP[i * 4 + k]);
                pMC->addParam(pA->m_vSlots[k], buf);
            }
            mModules[pA->getActionName()] = pMC;
        }
        int iResult = setPrioList();
        if (iResult == 0) iResult = m_prio.getActionAttributes(mModules);
        for (modulemap::iterator it = mModules.begin(); it != mModules.end(); ++it) delete it->second;
        setGpuCapacity(adK, (int)m_pCG->m_iNumCells);
        return iResult;
    }

    // the tutorial actions of GpuSexualPop, or the configured ones
    virtual int preLoop() {
        return m_bParamMode ? GpuPop<GpuSexualAgent>::preLoop() : GpuSexualPop::preLoop();
    }

    // genomes beside the agents, as Genetics::init sets them up
    // (actions/Genetics.cpp:205-213)
    void enableGenomes(int iGenomeSize, int iNumCrossover, double dMutationRate) {
        m_iWords = 2 * (uint)((iGenomeSize + 63) / 64);
        m_aGenomes.init(m_pAgentController->getLayerSize(), m_iWords);
        m_pAgentController->addBuffer(static_cast<LBBase *>(&m_aGenomes));
        setGpuGenetics(iGenomeSize, iNumCrossover, dMutationRate, &m_aGenomes);
    }

    void load(uint32_t N, const int64_t *id, const int32_t *cell, const float *birth, const float *age,
              const float *lastb, const uint8_t *gender, const uint8_t *state, const uint64_t *genome) {
        if (N == 0) return;
        const int iStart = (int)m_pAgentController->reserveSpace2(N);
        for (uint32_t i = 0; i < N; i++) {
            GpuSexualAgent &a = m_aAgents[iStart + (int)i];
            a.m_iLifeState = state[i];
            a.m_iCellIndex = cell[i];
            a.m_ulID = (idtype)id[i];
            a.m_ulCellID = m_pCG->m_aCells[cell[i]].m_iGlobalID;
            a.m_fBirthTime = birth[i];
            a.m_iGender = gender[i];
            a.m_fAge = age[i];
            a.m_fLastBirth = lastb[i];
            a.m_iMateIndex = -3;
            if (m_iWords > 0) memcpy(&m_aGenomes[(uint)(iStart + (int)i)], genome + (size_t)i * m_iWords,
                                     m_iWords * sizeof(uint64_t));
        }
    }

    void write(FILE *f) {
        std::vector<int64_t> id;
        std::vector<int32_t> cell;
        std::vector<float> birth, age, lastb;
        std::vector<uint8_t> gender, state;
        std::vector<uint64_t> genome;
        const int iFirst = getFirstAgentIndex();
        if (iFirst != LBController::NIL) {
            for (int iA = iFirst; iA <= getLastAgentIndex(); iA++) {
                const GpuSexualAgent &a = m_aAgents[iA];
                if (a.m_iLifeState <= 0) continue;
                id.push_back((int64_t)a.m_ulID);
                cell.push_back(a.m_iCellIndex);
                birth.push_back(a.m_fBirthTime);
                age.push_back(a.m_fAge);
                lastb.push_back(a.m_fLastBirth);
                gender.push_back(a.m_iGender);
                state.push_back((uint8_t)a.m_iLifeState);
                if (m_iWords > 0) {
                    const ulong *g = &m_aGenomes[(uint)iA];
                    genome.insert(genome.end(), g, g + m_iWords);
                }
            }
        }
        const uint64_t n = id.size();
        fwrite(&n, 8, 1, f);
        fwrite(id.data(), 8, n, f);
        fwrite(cell.data(), 4, n, f);
        fwrite(birth.data(), 4, n, f);
        fwrite(age.data(), 4, n, f);
        fwrite(lastb.data(), 4, n, f);
        fwrite(gender.data(), 1, n, f);
        fwrite(state.data(), 1, n, f);
        updateNumAgentsPerCell();
        const uint32_t C = (uint32_t)m_pCG->m_iNumCells;
        fwrite(&C, 4, 1, f);
        for (uint32_t c = 0; c < C; c++) {
            const uint32_t k = (uint32_t)m_aiNumAgentsPerCell[c];
            fwrite(&k, 4, 1, f);
        }
        fwrite(&m_iWords, 4, 1, f);
        fwrite(genome.data(), 8, genome.size(), f);
        int64_t iMinNext = -1;
        for (int t = 0; t < m_iNumThreads; t++) {
            IDGen g = *m_apIDGen[t];
            const int64_t iNext = (int64_t)g.getID();
            if ((iMinNext < 0) || (iNext < iMinNext)) iMinNext = iNext;
        }
        fwrite(&iMinNext, 8, 1, f);
    }

    uint m_iWords = 0;
    LayerArrBuf<ulong> m_aGenomes;
    bool m_bParamMode = false;
};

static bool rd(FILE *f, void *p, size_t sz, size_t n) { return (n == 0) || (fread(p, sz, n, f) == n); }

int main(int argc, char *argv[]) {
    if (argc < 3) return 2;
    const int iWriteEvery = (argc > 3) ? atoi(argv[3]) : 0;
    const bool bParam = (argc > 4) && (strcmp(argv[4], "param") == 0);
    FILE *fIn = fopen(argv[1], "rb");
    if (fIn == NULL) return 2;
    char magic[8];
    uint32_t C, N, nSteps, iLayer, nAct;
    uint64_t seed;
    bool ok = rd(fIn, magic, 1, 8) && (memcmp(magic, "QHGREF01", 8) == 0);
    ok = ok && rd(fIn, &C, 4, 1) && rd(fIn, &N, 4, 1) && rd(fIn, &nSteps, 4, 1) && rd(fIn, &iLayer, 4, 1);
    ok = ok && rd(fIn, &seed, 8, 1) && rd(fIn, &nAct, 4, 1);
    // the tutorial action set, parameters by type
    std::string sParams;
    char buf[256];
    std::vector<uint32_t> vType, vPrio;
    std::vector<double> vP;
    for (uint32_t i = 0; ok && (i < nAct); i++) {
        uint32_t type, prio;
        double p[4];
        ok = rd(fIn, &type, 4, 1) && rd(fIn, &prio, 4, 1) && rd(fIn, p, 8, 4);
        vType.push_back(type);
        vPrio.push_back(prio);
        vP.insert(vP.end(), p, p + 4);
        if (type == QHG_ACT_FERTILITY) {
            snprintf(buf, sizeof(buf), "Fertility_min_age=%.17g;Fertility_max_age=%.17g;Fertility_interbirth=%.17g;",
                     p[0], p[1], p[2]);
        } else if (type == QHG_ACT_VERHULST) {
            snprintf(buf, sizeof(buf), "Verhulst_b0=%.17g;Verhulst_d0=%.17g;Verhulst_theta=%.17g;Verhulst_K=%.17g;",
                     p[0], p[1], p[2], p[3]);
        } else if (type == QHG_ACT_RANDOMMOVE) {
            snprintf(buf, sizeof(buf), "RandomMove_prob=%.17g;", p[0]);
        } else {
            buf[0] = '\0';
        }
        sParams += buf;
    }
    uint32_t iGenome = 0, iDump = 0;
    int32_t iCross = 0;
    double dMut = 0;
    ok = ok && rd(fIn, &iGenome, 4, 1) && rd(fIn, &iCross, 4, 1) && rd(fIn, &dMut, 8, 1) && rd(fIn, &iDump, 4, 1);
    std::vector<int32_t> vNbr(ok ? (size_t)C * 6 : 0);
    std::vector<uint8_t> vNN(ok ? C : 0);
    std::vector<double> vK(ok ? C : 0);
    ok = ok && rd(fIn, vNbr.data(), 4, vNbr.size()) && rd(fIn, vNN.data(), 1, C) && rd(fIn, vK.data(), 8, C);
    std::vector<int64_t> vID(ok ? N : 0);
    std::vector<int32_t> vCell(ok ? N : 0);
    std::vector<float> vB(ok ? N : 0), vA(ok ? N : 0), vL(ok ? N : 0);
    std::vector<uint8_t> vG(ok ? N : 0), vS(ok ? N : 0);
    ok = ok && rd(fIn, vID.data(), 8, N) && rd(fIn, vCell.data(), 4, N) && rd(fIn, vB.data(), 4, N) &&
         rd(fIn, vA.data(), 4, N) && rd(fIn, vL.data(), 4, N) && rd(fIn, vG.data(), 1, N) && rd(fIn, vS.data(), 1, N);
    const size_t nWords = (iGenome > 0) ? (size_t)N * 2 * ((iGenome + 63) / 64) : 0;
    std::vector<uint64_t> vGen(ok ? nWords : 0);
    ok = ok && rd(fIn, vGen.data(), 8, nWords);
    // optional: u32 has_weights, f64 W[C*7]; u32 n_k_changes, (u32 step, f64 K[C])...
    uint32_t iHasW = 0, nKC = 0;
    std::vector<double> vW, vKC;
    std::vector<uint32_t> vKCStep;
    if (ok && rd(fIn, &iHasW, 4, 1)) {
        if (iHasW == 1) {
            vW.resize((size_t)C * 7);
            ok = rd(fIn, vW.data(), 8, vW.size());
        }
        ok = ok && rd(fIn, &nKC, 4, 1);
        vKCStep.resize(ok ? nKC : 0);
        vKC.resize(ok ? (size_t)nKC * C : 0);
        for (uint32_t k = 0; ok && (k < nKC); k++) {
            ok = rd(fIn, &vKCStep[k], 4, 1) && rd(fIn, vKC.data() + (size_t)k * C, 8, C);
        }
    }
    // optional: u32 movestats_mode + 1 (must be 0 here); u32 n_kill_events,
    // (u32 step, u8 flags[C])...: agents in flagged cells die before that step
    // u32 n_mods, (u32 step, u32 name_len, char name[], f64 value)...: runtime
    // edits through the Prioritizer before that step
    uint32_t iMS1 = 0, nKill = 0, nMods = 0;
    std::vector<uint32_t> vKillStep, vModStep;
    std::vector<uint8_t> vKill;
    std::vector<std::string> vModName;
    std::vector<double> vModValue;
    if (ok && rd(fIn, &iMS1, 4, 1)) {
        if (iMS1 != 0) ok = false;
        if (ok && rd(fIn, &nKill, 4, 1)) {
            vKillStep.resize(nKill);
            vKill.resize((size_t)nKill * C);
            for (uint32_t k = 0; ok && (k < nKill); k++) {
                ok = rd(fIn, &vKillStep[k], 4, 1) && rd(fIn, vKill.data() + (size_t)k * C, 1, C);
            }
            if (ok && rd(fIn, &nMods, 4, 1)) {
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
        }
    }
    fclose(fIn);
    if (!ok) {
        fprintf(stderr, "malformed input\n");
        return 2;
    }

    stringmap smSurf;
    smSurf[SURF_TYPE] = SURF_EQSAHEDRON;
    SCellGrid *pCG = new SCellGrid(0, C, smSurf);
    pCG->m_aCells = new SCell[C];
    for (uint32_t c = 0; c < C; c++) {
        pCG->m_aCells[c].m_iGlobalID = (gridtype)c;
        pCG->m_aCells[c].m_iNumNeighbors = vNN[c];
        for (int j = 0; j < 6; j++) pCG->m_aCells[c].m_aNeighbors[j] = vNbr[(size_t)c * 6 + j];
        pCG->m_mIDIndexes[c] = c;
    }
    int nThreads = omp_get_max_threads();
    IDGen **apIDG = new IDGen*[nThreads];
    for (int t = 0; t < nThreads; t++) apIDG[t] = new IDGen(0, t, nThreads);
    // GpuPop takes the run's seed from the first two state words
    uint32_t aulState[16] = {0};
    aulState[0] = (uint32_t)(seed & 0xffffffffu);
    aulState[1] = (uint32_t)(seed >> 32);
    static uint aiSeeds[NUM_SEEDS] = {0};

    DrivePop *pPop = new DrivePop(pCG, apIDG, aulState, aiSeeds);
    std::vector<double> vEnvK(vK);   // the environment's K array, rewritten by K changes
    if (bParam) {
        if (pPop->configureActions(vType, vPrio, vP, vK.data()) != 0) {
            fprintf(stderr, "configuration refused\n");
            return 3;
        }
        if ((iHasW == 1) || (nKC > 0)) {
            pPop->setGpuEnvironment((nKC > 0) ? vEnvK.data() : NULL, (iHasW == 1) ? vW.data() : NULL);
        }
    } else if (pPop->setParams(sParams) != 0) {
        fprintf(stderr, "setParams refused [%s]\n", sParams.c_str());
        return 3;
    }
    if (iGenome > 0) pPop->enableGenomes((int)iGenome, iCross, dMut);
    pPop->load(N, vID.data(), vCell.data(), vB.data(), vA.data(), vL.data(), vG.data(), vS.data(), vGen.data());
    if (pPop->preLoop() != 0) {
        fprintf(stderr, "preLoop failed: %s\n", pPop->gpuError());
        return 3;
    }
    std::set<uint> sPrios;
    for (uint32_t s = 0; s < nSteps; s++) {
        const float fT = (float)s;
        for (uint32_t k = 0; k < nKC; k++) {
            if (vKCStep[k] == s) {
                memcpy(vEnvK.data(), vKC.data() + (size_t)k * C, (size_t)C * sizeof(double));
                pPop->updateEvent(EVENT_ID_VEG, NULL, fT);
            }
        }
        for (uint32_t k = 0; k < nMods; k++) {
            if (vModStep[k] == s) pPop->modify(vModName[k], vModValue[k]);
        }
        for (uint32_t k = 0; k < nKill; k++) {
            if ((vKillStep[k] == s) && (pPop->removeAgentsInCells(vKill.data() + (size_t)k * C) != 0)) {
                fprintf(stderr, "removal failed\n");
                return 4;
            }
        }
        int iRes = pPop->initializeStep(fT);
        sPrios.clear();
        pPop->prios(sPrios);
        for (std::set<uint>::const_iterator it = sPrios.begin(); it != sPrios.end(); ++it) {
            iRes += pPop->doActions(*it, fT);
        }
        iRes += pPop->finalizeStep();
        if ((iWriteEvery > 0) && (((s + 1) % (uint32_t)iWriteEvery) == 0)) iRes += pPop->preWrite(fT);
        if (iRes != 0) {
            fprintf(stderr, "step %u failed\n", s);
            return 4;
        }
    }
    if (pPop->preWrite((float)nSteps) != 0) return 5;
    FILE *fOut = fopen(argv[2], "wb");
    if (fOut == NULL) return 2;
    pPop->write(fOut);
    fclose(fOut);
    return 0;
}
