/*
 * TEST INFRASTRUCTURE ONLY.  A stand-in for libqhg_gpu.so with the C ABI of
 * include/qhg_gpu.h, running each call on the oracle (oracle/qhg_oracle.c),
 * so that the population plugin's host code (qhg4_gb300/plugin: GpuPop<T>,
 * GpuSexualPop) can be run under a PopLooper-like loop on a machine without
 * a GPU.  tests/test_plugin_host.py builds it into a temporary directory as
 * libqhg_gpu.so for the plugin driver only; nothing else loads it.  Only the
 * calls the plugin makes are provided.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "qhg_gpu.h"

typedef struct qo_run qo_run;
qo_run *qo_create(uint64_t seed, int n_act, const int32_t *types, const double *params, int genome_size,
                  int num_crossover, double mutation_rate, int C, const int32_t *nbr, const uint8_t *nnbr,
                  const double *K);
int qo_load(qo_run *r, int64_t N, const int64_t *id, const int32_t *cell, const float *birth, const float *age,
            const float *lastb, const uint8_t *gender, const uint8_t *state, const uint64_t *genome,
            int32_t first_step);
int qo_step(qo_run *r, int nsteps, uint64_t *stats_out);
int64_t qo_num_agents(const qo_run *r);
int64_t qo_next_id(const qo_run *r);
void qo_set_next_id(qo_run *r, int64_t next_id);
int32_t qo_current_step(const qo_run *r);
int qo_get_agents(const qo_run *r, int64_t *id, int32_t *cell, float *birth, float *age, float *lastb,
                  uint8_t *gender, uint8_t *state, uint64_t *genome);
int qo_get_counts(const qo_run *r, uint32_t *counts);
int qo_set_capacity(qo_run *r, const double *K);
int qo_set_ice(qo_run *r, const uint8_t *ice);
int qo_set_move_weights(qo_run *r, const double *W);
void qo_destroy(qo_run *r);

struct qhg_run {
    qhg_run_desc desc;
    qo_run *o;
};

static const char *g_err = "";

const char *qhg_gpu_last_error(void) { return g_err; }

int qhg_gpu_create(const qhg_run_desc *desc, qhg_run **out) {
    if (desc == NULL || out == NULL || desc->n_actions < 0 || desc->n_actions > QHG_MAX_ACTIONS) {
        g_err = "bad arguments";
        return QHG_ERR_ARG;
    }
    qhg_run *r = (qhg_run *)calloc(1, sizeof(qhg_run));
    r->desc = *desc;
    *out = r;
    return QHG_OK;
}

int qhg_gpu_upload_grid(qhg_run *r, const int32_t *nbr6, const uint8_t *nnbr, const double *K, int32_t C) {
    if (r == NULL || C <= 0) return QHG_ERR_ARG;
    if (r->o != NULL) qo_destroy(r->o);
    r->o = qo_create(r->desc.seed, r->desc.n_actions, r->desc.action_type, &r->desc.action_param[0][0],
                     r->desc.genome_size, r->desc.num_crossover, r->desc.mutation_rate, C, nbr6, nnbr, K);
    if (r->o == NULL) {
        g_err = "oracle rejected the run";
        return QHG_ERR_ARG;
    }
    return QHG_OK;
}

int qhg_gpu_upload_agents(qhg_run *r, const qhg_agents_soa *a, int64_t n, int32_t first_step) {
    if (r == NULL || r->o == NULL) return QHG_ERR_STATE;
    return qo_load(r->o, n, a->id, a->cell, a->birth, a->age, a->last_birth, a->gender, a->state, a->genome,
                   first_step) == 0 ? QHG_OK : QHG_ERR_ARG;
}

int qhg_gpu_step(qhg_run *r, int32_t nsteps) {
    if (r == NULL || r->o == NULL) return QHG_ERR_STATE;
    qo_step(r->o, nsteps, NULL);
    return QHG_OK;
}

int qhg_gpu_num_agents(qhg_run *r, int64_t *n) {
    if (r == NULL || r->o == NULL) return QHG_ERR_STATE;
    *n = qo_num_agents(r->o);
    return QHG_OK;
}

int qhg_gpu_download(qhg_run *r, qhg_agents_soa *o, int64_t cap, int64_t *n) {
    if (r == NULL || r->o == NULL) return QHG_ERR_STATE;
    const int64_t k = qo_num_agents(r->o);
    if (k > cap) return QHG_ERR_CAPACITY;
    qo_get_agents(r->o, o->id, o->cell, o->birth, o->age, o->last_birth, o->gender, o->state, o->genome);
    *n = k;
    return QHG_OK;
}

int qhg_gpu_counts(qhg_run *r, uint32_t *counts) {
    if (r == NULL || r->o == NULL) return QHG_ERR_STATE;
    qo_get_counts(r->o, counts);
    return QHG_OK;
}

int qhg_gpu_set_capacity(qhg_run *r, const double *K) {
    if (r == NULL || r->o == NULL) return QHG_ERR_STATE;
    return qo_set_capacity(r->o, K) == 0 ? QHG_OK : QHG_ERR_ARG;
}

int qhg_gpu_set_move_weights(qhg_run *r, const double *W) {
    if (r == NULL || r->o == NULL) return QHG_ERR_STATE;
    return qo_set_move_weights(r->o, W) == 0 ? QHG_OK : QHG_ERR_ARG;
}


int qhg_gpu_set_ice(qhg_run *r, const uint8_t *ice) {
    if (r == NULL || r->o == NULL) return QHG_ERR_STATE;
    return qo_set_ice(r->o, ice) == 0 ? QHG_OK : QHG_ERR_ARG;
}

int qhg_gpu_next_id(qhg_run *r, int64_t *next_id) {
    if (r == NULL || r->o == NULL) return QHG_ERR_STATE;
    *next_id = qo_next_id(r->o);
    return QHG_OK;
}

int qhg_gpu_set_next_id(qhg_run *r, int64_t next_id) {
    if (r == NULL || r->o == NULL) return QHG_ERR_STATE;
    qo_set_next_id(r->o, next_id);
    return QHG_OK;
}

int qhg_gpu_current_step(qhg_run *r, int32_t *step) {
    if (r == NULL || r->o == NULL) return QHG_ERR_STATE;
    *step = qo_current_step(r->o);
    return QHG_OK;
}

int qhg_gpu_destroy(qhg_run *r) {
    if (r == NULL) return QHG_OK;
    if (r->o != NULL) qo_destroy(r->o);
    free(r);
    return QHG_OK;
}
