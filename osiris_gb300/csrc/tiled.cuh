// tiled.cuh -- particle engine with particles binned by spatial tile (single precision).
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"

namespace osg {

struct TiledState;

int tiled_create(TiledState **out, const osg_config &cfg, const GridDesc &g);
void tiled_destroy(TiledState *t);
int tiled_add_species(TiledState *t, double rqm, long np, const int *ix, const float *x,
                      const float *u, const float *q, cudaStream_t st);
// one push + deposit + migration pass over all species; parity selects which particle buffer
// is read (the other one is written)
// shift = 1: the step ends with a moving-window move (particles stored one cell lower in x1)
int tiled_push(TiledState *t, int parity, const float *e, const float *b, float *j,
               double *d_ene, int *d_status, cudaStream_t st, int *launches, int shift = 0);
// moving window along x1 at c: open x1 boundary for the particles, and injection of cold
// particles of `species` into the new last x1 plane with a piecewise-linear density profile
int tiled_set_window(TiledState *t, int species, const int *ppc, int nprof,
                     const double *prof_x, const double *prof_f);
int tiled_window_inject(TiledState *t, int parity, int *d_status, cudaStream_t st,
                        int *launches);
// the window's injection parameters (false: no window), and the device count of window moves
// (read by the injection) set to `moves` (restart)
bool tiled_window_params(const TiledState *t, int *species, int *ppc, int *nprof,
                         double *prof_x, double *prof_f);
int tiled_set_moves(TiledState *t, long moves, cudaStream_t st);
// `cur` = index (0/1) of the buffer that holds the current particles
int tiled_count(TiledState *t, int cur, int k, long *np, cudaStream_t st);
int tiled_get_species(TiledState *t, int cur, int k, int *ix, float *x, float *u, float *q,
                      cudaStream_t st);
int tiled_deposit_rho(TiledState *t, int cur, int k, double *rho, int *status,
                      cudaStream_t st);
// largest live-slot fraction over all tiles and species
int tiled_occupancy(TiledState *t, int cur, double *max_frac, cudaStream_t st);
// re-bin all species into larger slabs (host round trip); keeps buffer `cur` current
int tiled_regrow(TiledState *t, int cur, cudaStream_t st);

// pieces of tiled_push for the batched engine (many boxes per launch)
struct TiledArgs;
struct FoldBox;
struct IntRange;
TiledArgs tiled_args(TiledState *t, int parity, const float *e, const float *b, float *j,
                     double *d_ene, int *d_status);
FoldBox tiled_fold_box(TiledState *t, float *j);
IntRange tiled_arrival_counters(TiledState *t, int parity);
long tiled_ntiles(const TiledState *t);
size_t tiled_smem(const TiledState *t);
int tiled_threads(const TiledState *t);
// threads per push CTA (multiple of 32, 64..256); call before any step
int tiled_set_threads(TiledState *t, int threads);
// the thermal-bath random stream's step counter (device memory of the owner)
int tiled_set_step(TiledState *t, const unsigned long long *step);

} // namespace osg
