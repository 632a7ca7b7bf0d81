// Host-side helpers shared by the single-run API (qhg_api.cu) and the batch
// API (qhg_batch.cu): action constants, grid tables, launches.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "qhg_device.cuh"

int qhg_host_actions(qhg::StepConst &P, int n, const int32_t *types, const double (*params)[4], std::string &err);
int qhg_host_grid_tables(int C, const int32_t *nbr6, const uint8_t *nnbr, const double *K, bool wm,
                         const uint8_t *ice, std::vector<uint32_t> &rev, std::vector<uint64_t> &wthr,
                         std::vector<uint32_t> &cmove, std::string &err);
void qhg_host_ice_bits(int C, const int32_t *nbr6, const uint8_t *ice, std::vector<uint32_t> &cmove);
// MoveStats' distance from cell a to cell b (spherdistDeg / cartdist,
// utils/geomutils.cpp:311-386)
double qhg_host_move_distance(const double *lon, const double *lat, double radius, bool cartesian, int a, int b);
int qhg_host_move_tables(int C, const uint8_t *nnbr, const double *W, std::vector<uint64_t> &wthr,
                         std::vector<uint32_t> &cmove, std::string &err);

extern "C" int qhg_launch_refresh_cells(const qhg::StepConst *P, const qhg::RunState *rs, const uint32_t *nonempty,
                                        const uint32_t *ne_start, const double *K, const uint32_t *cmove,
                                        ulonglong2 *vthr, uint32_t *necm, int grid, cudaStream_t stream);
extern "C" int qhg_launch_ms_fill(uint32_t c0, uint32_t c1, int mode, const uint32_t *origin, uint32_t norigin,
                                  int32_t *hops, double *dist, double *time, int32_t *chops,
                                  unsigned long long *cdist, unsigned long long *ckey, double *D, cudaStream_t stream);
extern "C" int qhg_launch_grid_tables(int C, const int32_t *nbr6, const uint8_t *nnbr, const double *K, int wm,
                                      uint32_t *rev, uint32_t *cmove, double *W, uint64_t *wthr,
                                      unsigned long long *bad, int pass, cudaStream_t stream);
extern "C" int qhg_launch_refresh_cells_batch(const qhg::StepConst *P, const qhg::BatchRun *runs, const uint32_t *crun,
                                              const qhg::RunState *rs, const uint32_t *nonempty,
                                              const uint32_t *ne_start, const double *K, const uint32_t *cmove,
                                              ulonglong2 *vthr, uint32_t *necm, uint32_t cell0, uint32_t cell1,
                                              int grid, cudaStream_t stream);
extern "C" int qhg_launch_step(const qhg::StepConst *P, qhg::RunState *rs, const qhg::StepBuffers *B,
                               const qhg::BatchBuffers *BB, const qhg::LaunchShape *L, cudaStream_t stream);
extern "C" int qhg_launch_step_timed(const qhg::StepConst *P, qhg::RunState *rs, const qhg::StepBuffers *B,
                                     const qhg::BatchBuffers *BB, const qhg::LaunchShape *L, cudaStream_t stream,
                                     cudaEvent_t *ev);
extern "C" void qhg_tile_ctas_per_sm(int *actions, int *scatter);
extern "C" int qhg_match_program(const int32_t *types, int n);
extern "C" uint32_t qhg_program_window(int p, int a);

extern "C" int qhg_launch_batch_stage(uint32_t s0, uint32_t n, uint32_t cell0, uint32_t ncells, const int32_t *cell,
                                      uint8_t *smeta, const uint8_t *sgender, const int64_t *sid, uint32_t *scell,
                                      uint32_t *inj, unsigned long long *err, cudaStream_t stream);
extern "C" int qhg_launch_run_cells(const uint32_t *nonempty, const uint32_t *ne_start, uint32_t n_nonempty,
                                    uint32_t cell0, uint32_t cell1, uint32_t row0, uint32_t nrows,
                                    uint32_t *row_cell, uint32_t *counts, cudaStream_t stream);
