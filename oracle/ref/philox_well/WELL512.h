/*
 * Test-build replacement for the reference's utils/WELL512.h.
 *
 * ORACLE / TEST INFRASTRUCTURE ONLY.  oracle/ref/Makefile puts this
 * directory ahead of the reference's utils/ on the include path when it
 * builds the "Philox test build" of the reference (qhg_ref_philox).  The
 * reference's action code keeps calling m_apWELL[thread]->wrandd() etc.;
 * here every draw comes from a counter-based Philox4x32-10 stream that the
 * harness selects per (step, agent ID, action) through a thread-local
 * context, so results no longer depend on thread count or slot layout.
 *
 * The conversion formulas wrandd / wrandr / wrandi are the reference's
 * (utils/WELL512.h:33-39) and must stay identical to it: they define how a
 * 32-bit draw u becomes a double (u / 2^32), a range value and an index.
 */
#ifndef __WELL512_H__
#define __WELL512_H__

#include <cstdlib>
#include <cstdint>
#include <cstdio>
#include "qhg_consts.h"
#include "../../philox4x32.h"

static const unsigned int STATE_SIZE = 16;
static const unsigned long MAX_WRAND = 0xffffffff;

/* the stream the next draw comes from; set by the harness before it calls
 * into reference code that draws */
struct QhgDrawContext {
    uint64_t seed;
    uint32_t step;
    int64_t  id;
    uint32_t base;    /* first block of the stream */
    uint32_t next;    /* index of the next draw in the stream */
    uint32_t limit;   /* draws allowed in this window (window overflow is an error) */
    int      active;
};
extern thread_local QhgDrawContext g_qhgDrawCtx;
/* counts draws made outside a context or beyond a window; the harness
 * fails the run if it is nonzero */
extern unsigned long g_qhgDrawErrors;

class WELL512 {
public:
    WELL512(uint32_t *aulState, uint32_t uiIndex=0) { seed(aulState, uiIndex); }
    WELL512() : m_uiIndex(0), m_iCount(0) { for (unsigned i = 0; i < STATE_SIZE; i++) m_aulState[i] = 0; }
    ~WELL512() { }

    void seed(uint32_t *aulState, uint32_t uiIndex) {
        for (unsigned i = 0; i < STATE_SIZE; i++) m_aulState[i] = aulState[i];
        m_uiIndex = uiIndex;
        m_iCount = 0;
    }

    uint32_t wrand() {
        m_iCount++;
        QhgDrawContext &c = g_qhgDrawCtx;
        if (!c.active || c.next >= c.limit) {
            __atomic_fetch_add(&g_qhgDrawErrors, 1UL, __ATOMIC_RELAXED);
            return 0;
        }
        uint32_t k = c.next++;
        return qhg_oracle_draw(c.seed, c.step, c.id, c.base, k);
    }

    double   wrandd() { return (1.0*wrand())/(1+MAX_WRAND); };
    double   wrandr(double a, double b) { return a + ((b-a)*wrand())/(1+MAX_WRAND); };
    uint32_t wrandi(uint32_t a, uint32_t b, uint32_t s=1) { uint32_t r=b-a; r+=(r%s); return a+s*(uint32_t)((1.0*r*wrand())/(s*(1.0+MAX_WRAND))); };

    /* not on the hot path; drawing a Gaussian would consume an unknown
     * number of draws, so it is counted as an error */
    double   wgauss(double dSigma) { (void)dSigma; __atomic_fetch_add(&g_qhgDrawErrors, 1UL, __ATOMIC_RELAXED); return 0.0; }

    const uint32_t *getState() const { return m_aulState; }
    const uint32_t  getIndex() const { return m_uiIndex; }
    unsigned long   getCount() { return m_iCount; }
    double          getSigma() { return 0.0; }
    double          getPrevNormal() { return 0.0; }
    void setGaussStates(double dPrevNormal, double dSigma) { (void)dPrevNormal; (void)dSigma; }
    void showState() { }
    void state2String(char *pString) { if (pString) pString[0] = '\0'; }
    uint32_t getLastRand() { return 0; }
private:
    uint32_t      m_aulState[STATE_SIZE];
    uint32_t      m_uiIndex;
    unsigned long m_iCount;
};

#endif
