// tiled.cu -- single-precision particle engine with particles binned by spatial tile.
//
// Layout in HBM: for every species two particle buffers (ping-pong), each a set of SoA
// streams (cell index per axis, in-cell offset per axis, three momenta, charge) cut into
// fixed-capacity slabs, one slab per tile.  A slab holds the tile's particles sorted by cell in
// slots [0, cnt) and the particles that arrived from other tiles during the last step in slots
// [cap - arr, cap) (filled from the top).
//
// One push launch handles every species: CTA t owns tile t.  It stages E and B of the tile
// plus the stencil halo in shared memory and zeroes a shared current tile with its halo (one
// copy per warp in 2D).  Per species, every warp streams chunks of the tile's particles
// (coalesced SoA loads, the next chunk prefetched), gathers the fields from shared memory,
// does the Boris push, moves, trims and periodically wraps the particle, splits the trajectory
// at cell faces and accumulates the charge-conserving current of every segment into the shared
// tile (warp transpose-reduce per cell, or direct shared adds).  Particles that stay are
// written back to their own input slot and counted per cell; particles that leave are queued
// in shared memory and then appended to the arrival region of their destination tile in the
// other buffer.  A second pass counting-sorts the particles that stayed into the other buffer,
// so every step starts from cell-sorted tiles.  The shared current tile is added to the global
// current at the end (the halo overlaps the neighbours' halos).
//
// The per-particle arithmetic is the same as the plain engine (pic_math.cuh) and therefore the
// same as the reference kernels FNAME(vadvance_deposit_{2d,3d}_sN) (source/simd/
// os-spec-push-avx2.c:471-760, :1141-1480); only the order in which current contributions are
// summed differs.  The migration and the per-step tile sort replace both the periodic particle
// boundary (source/spec/os-spec-boundary.f03:1280-1290) and the cell sort every n_sort steps
// (source/spec/os-species.f03:269-505).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "fields.cuh"
#include "pic_math.cuh"
#include "push_plain.cuh"
#include "tiled.cuh"
#include "tile_ops.cuh"

namespace osg {

struct Slabs {
    int *ix[3];
    float *x[3];
    float *u[3];
    float *q;
    int *cnt;      // [ntiles] particles in slots [0, cnt) of the slab, sorted by cell
    int *arr;      // [ntiles] particles that arrived from other tiles, slots [cap - arr, cap)
};

struct SpeciesDev {
    Slabs in, out;
    float tem;
    int pad;
    long cap;      // slots per tile
};

struct TiledArgs {
    int T[3];          // tile shape (cells)
    int ntile[3];      // tiles per axis
    int nx[3];         // cells per axis
    int gcl[3];        // global guard cells (lower)
    int size[3];       // global grid extent incl. guards
    float dtdx[3];
    float jn[3];
    const float *e;
    const float *b;
    float *j;
    const SpeciesDev *spec;
    int nspec;
    double *ene;
    int *status;
    int reduce_min;    // warp-reduce a cell's segments when at least this many lanes share it
};

struct TiledState {
    int dim = 2, order = 2;
    int T[3] = {1, 1, 1}, ntile[3] = {1, 1, 1}, nx[3] = {1, 1, 1};
    long ntiles = 1;
    double capacity = 2.0;
    GridDesc g;
    double dt = 0, dx[3] = {1, 1, 1};
    std::vector<double> rqm;
    std::vector<long> cap;
    std::vector<Slabs> buf[2];
    std::vector<void *> allocs;
    int *d_cnt[2] = {nullptr, nullptr};   // [MAX_TILED_SPECIES * ntiles] per buffer
    SpeciesDev *d_tab[2] = {nullptr, nullptr};
    int *d_arr[2] = {nullptr, nullptr};   // arrival counters, [species][tile] per buffer
    int *d_off = nullptr;
    void *d_compact = nullptr;
    size_t compact_bytes = 0;
    size_t smem_bytes = 0;
    int threads = 256;   // threads per push CTA (multiple of 32, <= 256)
    int reduce_min = 2;  // set per dimension in tiled_create
};

static const int MAX_TILED_SPECIES = 16;
static const int MAX_TILE_CELLS = 1024;   // cells per tile (bins of the per-tile cell sort)

__device__ __forceinline__ int wrapc(int c, int n)
{
    return c < 1 ? c + n : (c > n ? c - n : c);
}

// In-place exclusive scan of n ints in shared memory by one warp; returns the total.
__device__ __forceinline__ int warp_exclusive_scan(int *c, int n)
{
    const int lane = threadIdx.x & 31, per = (n + 31) >> 5;
    const int lo = lane * per, hi = min(lo + per, n);
    int mine = 0;
    for (int k = lo; k < hi; k++) mine += c[k];
    int incl = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    int run = incl - mine;
    for (int k = lo; k < hi; k++) {
        const int v = c[k];
        c[k] = run;
        run += v;
    }
    return __shfl_sync(0xffffffffu, incl, 31);
}

// --------------------------------------------------------------------------------- push
static const int LEAVE_QUEUE = 256;   // particles per CTA and species queued for emigration

// Write a particle that left its tile into an arrival slot (from the top of the slab) of its
// destination tile in the output buffer.  The arrival region stays above the particles the
// destination keeps this step: those are at most its input particles.
template <int DIM>
__device__ __forceinline__ void emigrate(const SpeciesDev &sd, long cap, long dest,
                                         const int *cw, const float *xo, const float *un,
                                         float q, int *status)
{
    const int k = atomicAdd(sd.out.arr + dest, 1);
    const int room = (int)cap - sd.in.cnt[dest] - sd.in.arr[dest];
    if (k >= room) {
        atomicOr(status, OSG_STATUS_OVERFLOW);
        return;
    }
    const long o = dest * cap + cap - 1 - k;
#pragma unroll
    for (int d = 0; d < DIM; d++) {
        sd.out.ix[d][o] = cw[d];
        sd.out.x[d][o] = xo[d];
    }
    sd.out.u[0][o] = un[0];
    sd.out.u[1][o] = un[1];
    sd.out.u[2][o] = un[2];
    sd.out.q[o] = q;
}

// Every warp of the CTA runs its own pipeline over chunks of 32 particles of the tile, with no
// block barrier inside the particle loop: load, gather, Boris, move, split, write the particle
// to its new slot, then deposit the segments (round t takes the t-th segment of every lane).
// In 2D every warp accumulates into its own copy of the current tile, so the warp-reduced
// passes add with plain shared read-modify-writes; the copies are summed when the tile is
// flushed.  In 3D the warps share one current tile (atomic adds).
// CTAs of up to 256 threads.  2D linear/quadratic: three resident CTAs per SM (at most 85
// registers per thread, measured fastest on GB300); 2D quartic: one (it needs ~250 registers
// without spilling); otherwise two
template <int DIM, int ORD>
constexpr int push_min_blocks() { return DIM == 2 ? (ORD <= 2 ? 3 : (ORD == 3 ? 2 : 1)) : 2; }

template <int DIM, int ORD>
__global__ void __launch_bounds__(256, push_min_blocks<DIM, ORD>()) k_push_tiled(TiledArgs a)
{
    constexpr int NP = ORD + 1, OFS = Stencil<ORD>::OFS;
    constexpr int MAXSEG = DIM == 2 ? 3 : 4;
    constexpr bool PRIV = private_current<DIM>();
    extern __shared__ float smem[];
    const long tile = blockIdx.x;
    int t0[3], tc[3];
    tc[0] = (int)(tile % a.ntile[0]);
    tc[1] = DIM > 1 ? (int)((tile / a.ntile[0]) % a.ntile[1]) : 0;
    tc[2] = DIM > 2 ? (int)(tile / ((long)a.ntile[0] * a.ntile[1])) : 0;
#pragma unroll
    for (int d = 0; d < 3; d++) t0[d] = tc[d] * a.T[d] + 1;

    // shared layout: E and B over ee points per axis, J over je points per axis, 3 comps each
    int ee[3], je[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        ee[d] = d < DIM ? a.T[d] + NP : 1;
        je[d] = d < DIM ? a.T[d] + NP + 1 : 1;
    }
    const int ne = ee[0] * ee[1] * ee[2], nj = je[0] * je[1] * je[2];
    const int nthr = blockDim.x, nwarp = nthr >> 5, warp = threadIdx.x >> 5;
    const int njall = 3 * nj * (PRIV ? nwarp : 1);
    float *sE = smem, *sB = smem + 3 * ne, *sJ = smem + 6 * ne;
    const long gsy = 3L * a.size[0], gsz = 3L * a.size[0] * a.size[1];

    // stage fields: local point l <-> Fortran cell t0 - OFS + l <-> global position
    // t0 - OFS + l - 1 + gcl (inside the guard cells for tiles at the box edge)
    for (int idx = threadIdx.x; idx < 3 * ne; idx += nthr) {
        const int c = idx % 3, pnt = idx / 3;
        const int lx = pnt % ee[0], ly = (pnt / ee[0]) % ee[1], lz = pnt / (ee[0] * ee[1]);
        long gp = 3L * (t0[0] - OFS + lx - 1 + a.gcl[0]) + c;
        if (DIM > 1) gp += gsy * (t0[1] - OFS + ly - 1 + a.gcl[1]);
        if (DIM > 2) gp += gsz * (t0[2] - OFS + lz - 1 + a.gcl[2]);
        sE[idx] = __ldg(a.e + gp);
        sB[idx] = __ldg(a.b + gp);
    }
    for (int idx = threadIdx.x; idx < njall; idx += nthr) sJ[idx] = 0.0f;
    __syncthreads();

    const int esy = 3 * ee[0], esz = 3 * ee[0] * ee[1];
    const int jsy = 3 * je[0], jsz = 3 * je[0] * je[1];
    const unsigned lane = threadIdx.x & 31;
    float *sJw = PRIV ? sJ + 3 * nj * warp : sJ;
    LaneSlots<DIM, ORD> ls;
    ls.init(jsy, jsz);
    // 3D direct deposits: every thread walks its own contiguous run of the cell-sorted tile,
    // so the lanes of a warp sit in cells far apart and their shared-memory atomics seldom
    // conflict; otherwise a warp takes 32 consecutive particles (mostly one cell)
    const bool spread = DIM == 3 && (direct_only<DIM, ORD>() || a.reduce_min > 32);

    __shared__ int sHist[MAX_TILE_CELLS];
    // particles leaving the tile wait in a shared queue; after the pass they take their
    // arrival slots all at once, so no warp waits on a global atomic inside the pass
    __shared__ int sLeaveI[LEAVE_QUEUE][4];      // new cell per axis, destination tile
    __shared__ float sLeaveF[LEAVE_QUEUE][8];    // offsets per axis, momenta, charge
    __shared__ int sNleave;
    // 2D: per-warp queues of segments for full-warp deposits (dynamic shared memory after the
    // current tile, 16-byte aligned)
    SegRec *sQ = reinterpret_cast<SegRec *>(smem + ((6 * ne + njall + 3) & ~3)) + warp * SEGQ;
    int qn = 0;
    const int ncell = a.T[0] * a.T[1] * a.T[2];

    for (int s = 0; s < a.nspec; s++) {
        const SpeciesDev sd = a.spec[s];
        const long cap = sd.cap;
        const long slab = tile * cap;
        const int nst = min(sd.in.cnt[tile], (int)cap);
        const int nar = min(sd.in.arr[tile], (int)cap - nst);
        const int n = nst + nar;
        for (int k = threadIdx.x; k < ncell; k += nthr) sHist[k] = 0;
        if (threadIdx.x == 0) sNleave = 0;
        __syncthreads();
        // per-thread partial energy in FP32 (the reference sums in single precision per
        // 464-particle chunk), summed over the block in double
        float my_ene = 0.f;
        // ---- pass A: push every particle of the tile.  Particles that stay are written back
        //      to their own slot of the input slab (this CTA owns it) and counted per new cell;
        //      particles that leave take an arrival slot (from the top) of their destination
        //      tile in the output buffer, and their input slot is marked empty (ix = 0).
        auto slot = [&](int i) { return slab + (i < nst ? i : cap - 1 - (i - nst)); };
        // the particle of the next iteration is loaded while this one is pushed
        int pf_c[3] = {1, 1, 1};
        float pf_x[3] = {0, 0, 0}, pf_u[3] = {0, 0, 0}, pf_q = 0.0f;
        auto prefetch = [&](int i, int lim) {
            if (i < lim) {
                const long p = slot(i);
#pragma unroll
                for (int d = 0; d < DIM; d++) {
                    pf_c[d] = sd.in.ix[d][p];
                    pf_x[d] = sd.in.x[d][p];
                }
                pf_u[0] = sd.in.u[0][p];
                pf_u[1] = sd.in.u[1][p];
                pf_u[2] = sd.in.u[2][p];
                pf_q = sd.in.q[p];
            }
        };
        // take the prefetched particle into registers
        auto take = [&](int *c, float *xo, float *un, float &q) {
#pragma unroll
            for (int d = 0; d < 3; d++) {
                c[d] = pf_c[d];
                xo[d] = pf_x[d];
                un[d] = pf_u[d];
            }
            q = pf_q;
        };
        // Push one particle (slot p; has = false: an idle lane), split its motion into in-cell
        // segments sg[0..nseg), and write it back (stays in the tile) or queue it (leaves).
        // Returns nseg, or -1 for an idle lane.  Warp-collective: every lane calls it.
        auto push_one = [&](bool has, long p, int *c, float *xo, float *un, float q,
                            SegRec *sg) -> int {
            int di[3] = {0, 0, 0};
            float x1[3] = {0, 0, 0};
            if (has) {
                bool ok = true;
#pragma unroll
                for (int d = 0; d < DIM; d++) {
                    const int lc = c[d] - t0[d];
                    ok = ok && lc >= 0 && lc < a.T[d];
                }
                if (!ok) {
                    atomicOr(a.status, OSG_STATUS_RANGE);
                    sd.in.ix[0][p] = 0;
                    has = false;
                }
            }
            // ---- gather from the staged tile, Boris, move, split into segments
            int nseg = 0;
            if (has) {
                float w[DIM][NP], wh[DIM][NP];
                int lf[DIM], lh[DIM];
#pragma unroll
                for (int d = 0; d < DIM; d++) {
                    spline<ORD>(xo[d], w[d]);
                    const bool neg = xo[d] < 0.0f;
                    lf[d] = c[d] - t0[d] + 1;
                    lh[d] = lf[d] - (neg ? 1 : 0);
                    spline_h<ORD>(xo[d], neg ? 1.0f : 0.0f, wh[d]);
                }
                float E1, E2, E3, B1, B2, B3;
                gather_tile<DIM, ORD>(sE, sB, esy, esz, lf, lh, w, wh, E1, E2, E3, B1, B2, B3);
                const float ene = boris(sd.tem, E1, E2, E3, B1, B2, B3, un[0], un[1], un[2]);
                my_ene = fmaf(q, ene, my_ene);
                const float rg = rgamma(un[0], un[1], un[2]);
                const float vv[3] = {un[0] * rg, un[1] * rg, un[2] * rg};
#pragma unroll
                for (int d = 0; d < DIM; d++) {
                    x1[d] = fmaf(vv[d], a.dtdx[d], xo[d]);
                    di[d] = trim(x1[d]);
                }
                nseg = make_segments<DIM>(sg, xo, x1, di, vv[2], q, c[0] - t0[0] + 1,
                                          c[1] - t0[1] + 1, DIM > 2 ? c[2] - t0[2] + 1 : 0,
                                          jsy, jsz);
            }
            // ---- new position, cell (periodically wrapped) and destination tile
            long dest = -1;
            int cw[3] = {1, 1, 1};
            if (has) {
                long dt = 0, mul = 1;
#pragma unroll
                for (int d = 0; d < DIM; d++) {
                    xo[d] = x1[d] - float(di[d]);
                    cw[d] = wrapc(c[d] + di[d], a.nx[d]);
                    dt += mul * ((cw[d] - 1) / a.T[d]);
                    mul *= a.ntile[d];
                }
                dest = dt;
            }
            const bool stay = has && dest == tile;
            int lcell = -1;
            if (stay) {
#pragma unroll
                for (int d = 0; d < DIM; d++) {
                    sd.in.ix[d][p] = cw[d];
                    sd.in.x[d][p] = xo[d];
                }
                sd.in.u[0][p] = un[0];
                sd.in.u[1][p] = un[1];
                sd.in.u[2][p] = un[2];
                lcell = cw[0] - t0[0];
                if (DIM > 1) lcell += a.T[0] * (cw[1] - t0[1]);
                if (DIM > 2) lcell += a.T[0] * a.T[1] * (cw[2] - t0[2]);
            }
            const unsigned peers = __match_any_sync(FULL_MASK, lcell);
            if (stay && (int)lane == __ffs(peers) - 1) atomicAdd(&sHist[lcell], __popc(peers));
            const bool leave = has && !stay;
            const unsigned ml = __ballot_sync(FULL_MASK, leave);
            if (ml) {
                const int leader = __ffs(ml) - 1;
                int q0 = 0;
                if ((int)lane == leader) q0 = atomicAdd(&sNleave, __popc(ml));
                q0 = __shfl_sync(FULL_MASK, q0, leader);
                if (leave) {
                    sd.in.ix[0][p] = 0;
                    const int e = q0 + __popc(ml & ((1u << lane) - 1u));
                    if (e < LEAVE_QUEUE) {
#pragma unroll
                        for (int d = 0; d < 3; d++) {
                            sLeaveI[e][d] = cw[d];
                            sLeaveF[e][d] = xo[d];
                            sLeaveF[e][3 + d] = un[d];
                        }
                        sLeaveI[e][3] = (int)dest;
                        sLeaveF[e][6] = q;
                    } else {
                        emigrate<DIM>(sd, cap, dest, cw, xo, un, q, a.status);
                    }
                }
            }
            return has ? nseg : -1;
        };
        const int nit = (n + nthr - 1) / nthr;
        auto index = [&](int it) {
            return spread ? (int)threadIdx.x * nit + it : it * nthr + (int)threadIdx.x;
        };
        prefetch(index(0), n);
        for (int it = 0; it < nit; it++) {
            const int i = index(it);
            SegRec sg[MAXSEG];
            int c[3];
            float xo[3], un[3], q;
            take(c, xo, un, q);
            if (it + 1 < nit) prefetch(index(it + 1), n);
            const int ns = push_one(i < n, slot(i), c, xo, un, q, sg);
            // ---- charge-conserving current of the segments into the shared tile.  The first
            //      segment (in the particle's own cell, shared by neighbouring lanes of the
            //      cell-sorted tile) is warp-reduced per cell; in 2D the others (face
            //      crossings, few and scattered) wait in the warp's queue for a full-warp,
            //      cell-sorted deposit
#pragma unroll
            for (int t = 0; t < MAXSEG; t++) {
                const bool hs = t < ns;
                if (DIM == 2 && t > 0) {
                    segq_push(sQ, qn, hs, sg[t]);
                    if (qn >= 32) segq_drain<ORD>(sJw, sQ, qn, 32, a.jn, jsy);
                    continue;
                }
                if (!__any_sync(FULL_MASK, hs)) break;
                deposit_segment<DIM, ORD>(sJw, hs ? &sg[t] : nullptr, a.jn, jsy, jsz,
                                          a.reduce_min, ls);
            }
        }
        if (DIM == 2) segq_drain<ORD>(sJw, sQ, qn, 1, a.jn, jsy);
        const double tot = block_sum((double)my_ene);   // (contains block barriers)
        if (threadIdx.x == 0 && tot != 0.0) atomicAdd(a.ene + s, tot);
        // ---- the queued particles that left take their arrival slots
        {
            const int nq = min(sNleave, LEAVE_QUEUE);
            for (int e = threadIdx.x; e < nq; e += nthr) {
                int cw[3];
                float xo[3], un[3];
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    cw[d] = sLeaveI[e][d];
                    xo[d] = sLeaveF[e][d];
                    un[d] = sLeaveF[e][3 + d];
                }
                emigrate<DIM>(sd, cap, sLeaveI[e][3], cw, xo, un, sLeaveF[e][6], a.status);
            }
        }
        // ---- cell offsets of the particles that stayed
        if (threadIdx.x < 32) {
            const int nstay = warp_exclusive_scan(sHist, ncell);
            if (threadIdx.x == 0) sd.out.cnt[tile] = nstay;
        }
        __syncthreads();
        // ---- pass B: counting-sort the particles that stayed into the output slab, so that
        //      every step starts from particles in cell order (consecutive lanes share a cell)
        for (int base = 0; base < n; base += nthr) {
            const int i = base + threadIdx.x;
            const long p = slab + (i < nst ? i : cap - 1 - (i - nst));
            int lcell = -1;
            int cc[3] = {0, 0, 0};
            if (i < n) {
#pragma unroll
                for (int d = 0; d < DIM; d++) cc[d] = sd.in.ix[d][p];
                if (cc[0] != 0) {
                    lcell = cc[0] - t0[0];
                    if (DIM > 1) lcell += a.T[0] * (cc[1] - t0[1]);
                    if (DIM > 2) lcell += a.T[0] * a.T[1] * (cc[2] - t0[2]);
                }
            }
            const unsigned peers = __match_any_sync(FULL_MASK, lcell);
            const int leader = __ffs(peers) - 1;
            int first = 0;
            if (lcell >= 0 && (int)lane == leader) first = atomicAdd(&sHist[lcell], __popc(peers));
            first = __shfl_sync(FULL_MASK, first, leader);
            if (lcell >= 0) {
                const long o = slab + first + __popc(peers & ((1u << lane) - 1u));
#pragma unroll
                for (int d = 0; d < DIM; d++) {
                    sd.out.ix[d][o] = cc[d];
                    sd.out.x[d][o] = sd.in.x[d][p];
                }
                sd.out.u[0][o] = sd.in.u[0][p];
                sd.out.u[1][o] = sd.in.u[1][p];
                sd.out.u[2][o] = sd.in.u[2][p];
                sd.out.q[o] = sd.in.q[p];
            }
        }
        __syncthreads();
    }
    // ---- add the shared current tile (with halo; summed over the warp copies in 2D) to the
    //      global current
    for (int idx = threadIdx.x; idx < 3 * nj; idx += nthr) {
        float v = sJ[idx];
        if (PRIV)
            for (int w = 1; w < nwarp; w++) v += sJ[3 * nj * w + idx];
        if (v == 0.0f) continue;
        const int c = idx % 3, pnt = idx / 3;
        const int lx = pnt % je[0], ly = (pnt / je[0]) % je[1], lz = pnt / (je[0] * je[1]);
        long gp = 3L * (t0[0] - OFS + lx - 1 + a.gcl[0]) + c;
        if (DIM > 1) gp += gsy * (t0[1] - OFS + ly - 1 + a.gcl[1]);
        if (DIM > 2) gp += gsz * (t0[2] - OFS + lz - 1 + a.gcl[2]);
        atomicAdd(a.j + gp, v);
    }
}

// --------------------------------------------------------------------------------- binning
// scatter particles (reference layout) to precomputed slab slots (host counting sort by tile
// and by cell inside the tile)
__global__ void k_bin(const int *__restrict__ ix, const float *__restrict__ x,
                      const float *__restrict__ u, const float *__restrict__ q,
                      const long *__restrict__ dst, long np, int dim, Slabs out)
{
    OSG_GRID_LOOP(p, np)
    {
        const long o = dst[p];
        for (int d = 0; d < dim; d++) {
            out.ix[d][o] = ix[dim * p + d];
            out.x[d][o] = x[dim * p + d];
        }
        out.u[0][o] = u[3 * p];
        out.u[1][o] = u[3 * p + 1];
        out.u[2][o] = u[3 * p + 2];
        out.q[o] = q[p];
    }
}

// slab -> reference layout (ix(dim,N), x(dim,N), p(3,N), q(N)) at offsets off[tile]
__global__ void k_compact(Slabs in, long cap, int dim, const int *__restrict__ off, int *ix,
                          float *x, float *u, float *q)
{
    const long t = blockIdx.x;
    const int nst = min(in.cnt[t], (int)cap), n = nst + min(in.arr[t], (int)cap - nst);
    const long o = off[t];
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const long src = t * cap + (i < nst ? i : cap - 1 - (i - nst)), dst = o + i;
        for (int d = 0; d < dim; d++) {
            ix[dim * dst + d] = in.ix[d][src];
            x[dim * dst + d] = in.x[d][src];
        }
        u[3 * dst] = in.u[0][src];
        u[3 * dst + 1] = in.u[1][src];
        u[3 * dst + 2] = in.u[2][src];
        q[dst] = in.q[src];
    }
}

// --------------------------------------------------------------------------------- host
// The single-precision reference hands the push a time step rounded to p_k_part
// (dtcycle = real(dt, p_k_part), source/spec/os-spec-vpush.f03:365); the field solver keeps
// the double value.
static double push_dt(const TiledState *t) { return (double)(float)t->dt; }

static TiledArgs base_args(const TiledState *t)
{
    TiledArgs a;
    memset(&a, 0, sizeof a);
    const double dtp = push_dt(t);
    for (int d = 0; d < 3; d++) {
        a.T[d] = t->T[d];
        a.ntile[d] = t->ntile[d];
        a.nx[d] = t->nx[d];
        a.gcl[d] = t->g.gcl[d];
        a.size[d] = t->g.size[d];
        a.dtdx[d] = d < t->dim ? (float)(dtp / t->dx[d]) : 0.0f;
        const double div = t->dim == 2 ? 2.0 : 3.0;
        a.jn[d] = d < t->dim ? (float)(t->dx[d] / dtp / div) : 0.0f;
    }
    return a;
}

// shared memory of the push kernel: E and B tiles and the current tile (one per warp in 2D)
static size_t smem_for(int dim, int order, const int *T, int threads)
{
    const int NP = order + 1;
    size_t ne = 1, nj = 1;
    for (int d = 0; d < dim; d++) {
        ne *= (size_t)(T[d] + NP);
        nj *= (size_t)(T[d] + NP + 1);
    }
    const size_t copies = dim == 2 ? (size_t)threads / 32 : 1;
    const size_t nf = (6 * ne + 3 * nj * copies + 3) & ~(size_t)3;
    const size_t queues = dim == 2 ? (size_t)(threads / 32) * SEGQ * sizeof(SegRec) : 0;
    return nf * sizeof(float) + queues;
}

int tiled_create(TiledState **out, const osg_config &cfg, const GridDesc &g)
{
    TiledState *t = new TiledState();
    t->dim = cfg.dim;
    t->order = cfg.order;
    t->g = g;
    t->dt = cfg.dt;
    t->capacity = cfg.capacity > 0 ? cfg.capacity : 3.0;
    t->ntiles = 1;
    for (int d = 0; d < 3; d++) {
        t->nx[d] = d < cfg.dim ? cfg.nx[d] : 1;
        t->dx[d] = cfg.dx[d];
        int T = 1;
        if (d < cfg.dim) {
            T = cfg.tile[d];
            if (T <= 0) {
                const int pref = 8;   // measured best on GB300 for 2D quadratic (C2)
                for (T = pref; T > 1 && t->nx[d] % T; T >>= 1) {}
            }
            if (T < 1 || t->nx[d] % T) {
                delete t;
                set_error("tile size %d does not divide nx[%d] = %d", T, d, t->nx[d]);
                return OSG_ERR_ARG;
            }
        }
        t->T[d] = T;
        t->ntile[d] = t->nx[d] / T;
        t->ntiles *= t->ntile[d];
    }
    if (t->ntiles >= (1L << 30)) {
        set_error("too many tiles (%ld)", t->ntiles);
        delete t;
        return OSG_ERR_ARG;
    }
    if ((long)t->T[0] * t->T[1] * t->T[2] > MAX_TILE_CELLS) {
        set_error("a tile may hold at most %d cells", MAX_TILE_CELLS);
        delete t;
        return OSG_ERR_ARG;
    }
    // 2D: warp-reduce every cell that two or more lanes share; 3D (54..300 values per segment,
    // lanes of one warp spread over the tile): direct shared atomics measured faster
    t->reduce_min = t->dim == 2 ? 2 : 33;
    if (const char *ev = getenv("OSG_REDUCE_MIN")) t->reduce_min = atoi(ev);
    if (const char *ev = getenv("OSG_PUSH_THREADS")) {
        const int v = atoi(ev);
        if (v >= 64 && v <= 256 && v % 32 == 0) t->threads = v;
    }
    t->smem_bytes = smem_for(t->dim, t->order, t->T, t->threads);
    if (t->smem_bytes > 200 * 1024) {
        set_error("tile too large for shared memory (%zu bytes)", t->smem_bytes);
        delete t;
        return OSG_ERR_ARG;
    }
    // opt in to more than 48 KB of dynamic shared memory (outside any stream capture)
    {
        cudaError_t ce = cudaSuccess;
#define OSG_TATTR(D, O)                                                                       \
        if (t->dim == D && t->order == O)                                                     \
            ce = cudaFuncSetAttribute(k_push_tiled<D, O>,                                     \
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,            \
                                      (int)t->smem_bytes);
        OSG_TATTR(2, 1) OSG_TATTR(2, 2) OSG_TATTR(2, 3) OSG_TATTR(2, 4)
        OSG_TATTR(3, 1) OSG_TATTR(3, 2) OSG_TATTR(3, 3) OSG_TATTR(3, 4)
#undef OSG_TATTR
        if (ce != cudaSuccess) {
            set_error("cudaFuncSetAttribute: %s", cudaGetErrorString(ce));
            delete t;
            return OSG_ERR_CUDA;
        }
    }
    for (int p = 0; p < 2; p++) {
        if (cudaMalloc(&t->d_cnt[p], sizeof(int) * MAX_TILED_SPECIES * t->ntiles) != cudaSuccess ||
            cudaMalloc(&t->d_arr[p], sizeof(int) * MAX_TILED_SPECIES * t->ntiles) != cudaSuccess ||
            cudaMalloc(&t->d_tab[p], sizeof(SpeciesDev) * MAX_TILED_SPECIES) != cudaSuccess) {
            tiled_destroy(t);
            set_error("tile count allocation failed");
            return OSG_ERR_NOMEM;
        }
        cudaMemset(t->d_cnt[p], 0, sizeof(int) * MAX_TILED_SPECIES * t->ntiles);
        cudaMemset(t->d_arr[p], 0, sizeof(int) * MAX_TILED_SPECIES * t->ntiles);
    }
    if (cudaMalloc(&t->d_off, sizeof(int) * t->ntiles) != cudaSuccess) {
        tiled_destroy(t);
        set_error("offset allocation failed");
        return OSG_ERR_NOMEM;
    }
    *out = t;
    return OSG_OK;
}

void tiled_destroy(TiledState *t)
{
    if (!t) return;
    for (void *p : t->allocs) cudaFree(p);
    for (int p = 0; p < 2; p++) {
        cudaFree(t->d_cnt[p]);
        cudaFree(t->d_arr[p]);
        cudaFree(t->d_tab[p]);
    }
    cudaFree(t->d_off);
    cudaFree(t->d_compact);
    delete t;
}

static int upload_tables(TiledState *t, cudaStream_t st)
{
    const int ns = (int)t->rqm.size();
    for (int p = 0; p < 2; p++) {
        std::vector<SpeciesDev> tab(ns);
        for (int k = 0; k < ns; k++) {
            tab[k].in = t->buf[p][k];
            tab[k].out = t->buf[1 - p][k];
            tab[k].tem = (float)(0.5 * push_dt(t) / (double)(float)t->rqm[k]);
            tab[k].pad = 0;
            tab[k].cap = t->cap[k];
        }
        OSG_CUDA(cudaMemcpyAsync(t->d_tab[p], tab.data(), sizeof(SpeciesDev) * ns,
                                 cudaMemcpyHostToDevice, st));
    }
    OSG_CUDA(cudaStreamSynchronize(st));
    return OSG_OK;
}

int tiled_add_species(TiledState *t, double rqm, long np, const int *ix, const float *x,
                      const float *u, const float *q, cudaStream_t st)
{
    const int k = (int)t->rqm.size();
    OSG_CHECK(k < MAX_TILED_SPECIES, OSG_ERR_ARG, "too many species for the tiled engine");
    const int dim = t->dim;
    // key of every particle: tile, then cell inside the tile (x fastest)
    const long cells_per_tile = (long)t->T[0] * t->T[1] * t->T[2];
    std::vector<long> key(np);
    std::vector<int> cnt(t->ntiles, 0);
    for (long p = 0; p < np; p++) {
        long tt = 0, mul = 1, lc = 0, lmul = 1;
        for (int d = 0; d < dim; d++) {
            const int c = ix[dim * p + d] - 1;
            tt += mul * (c / t->T[d]);
            mul *= t->ntile[d];
            lc += lmul * (c % t->T[d]);
            lmul *= t->T[d];
        }
        key[p] = tt * cells_per_tile + lc;
        cnt[tt]++;
    }
    // slots per tile: capacity x mean load, and at least 1.25 x the initial maximum
    const int cmax = np > 0 ? *std::max_element(cnt.begin(), cnt.end()) : 0;
    const double mean = (double)np / (double)t->ntiles;
    long cap = (long)std::ceil(std::max(t->capacity * mean, 1.25 * cmax)) + 64;
    cap = (cap + 31) / 32 * 32;
    // stable counting sort by key -> slab slot of every particle
    std::vector<long> dst(np);
    {
        std::vector<long> off(t->ntiles * cells_per_tile + 1, 0);
        for (long p = 0; p < np; p++) off[key[p] + 1]++;
        for (size_t k = 1; k < off.size(); k++) off[k] += off[k - 1];
        std::vector<long> tile_first(t->ntiles);
        for (long tt = 0; tt < t->ntiles; tt++) tile_first[tt] = off[tt * cells_per_tile];
        for (long p = 0; p < np; p++) {
            const long k = key[p], tt = k / cells_per_tile;
            const long rank = off[k]++ - tile_first[tt];
            dst[p] = tt * cap + rank;
        }
    }
    const size_t nslot = (size_t)cap * t->ntiles;
    for (int p = 0; p < 2; p++) {
        Slabs s;
        memset(&s, 0, sizeof s);
        const size_t bytes = nslot * sizeof(float) * (2 * dim + 4);
        char *mem = nullptr;
        if (cudaMalloc(&mem, bytes) != cudaSuccess) {
            set_error("particle slab allocation of %zu bytes failed", bytes);
            return OSG_ERR_NOMEM;
        }
        t->allocs.push_back(mem);
        size_t o = 0;
        for (int d = 0; d < dim; d++) {
            s.ix[d] = (int *)(mem + o); o += nslot * 4;
        }
        for (int d = 0; d < dim; d++) {
            s.x[d] = (float *)(mem + o); o += nslot * 4;
        }
        for (int c = 0; c < 3; c++) {
            s.u[c] = (float *)(mem + o); o += nslot * 4;
        }
        s.q = (float *)(mem + o);
        s.cnt = t->d_cnt[p] + (size_t)k * t->ntiles;
        s.arr = t->d_arr[p] + (size_t)k * t->ntiles;
        OSG_CUDA(cudaMemsetAsync(s.arr, 0, sizeof(int) * t->ntiles, st));
        t->buf[p].push_back(s);
    }
    t->rqm.push_back(rqm);
    t->cap.push_back(cap);
    // upload in reference layout, bin into buffer 0
    if (np > 0) {
        const size_t need = (size_t)np * (sizeof(int) * dim + sizeof(float) * (dim + 4));
        if (need > t->compact_bytes) {
            cudaFree(t->d_compact);
            t->d_compact = nullptr;
            t->compact_bytes = 0;
            OSG_CUDA(cudaMalloc(&t->d_compact, need));
            t->compact_bytes = need;
        }
        int *dix = (int *)t->d_compact;
        float *dx_ = (float *)(dix + (size_t)dim * np);
        float *du = dx_ + (size_t)dim * np;
        float *dq = du + (size_t)3 * np;
        OSG_CUDA(cudaMemcpyAsync(dix, ix, sizeof(int) * dim * np, cudaMemcpyHostToDevice, st));
        OSG_CUDA(cudaMemcpyAsync(dx_, x, sizeof(float) * dim * np, cudaMemcpyHostToDevice, st));
        OSG_CUDA(cudaMemcpyAsync(du, u, sizeof(float) * 3 * np, cudaMemcpyHostToDevice, st));
        OSG_CUDA(cudaMemcpyAsync(dq, q, sizeof(float) * np, cudaMemcpyHostToDevice, st));
        OSG_CUDA(cudaMemcpyAsync(t->buf[0][k].cnt, cnt.data(), sizeof(int) * t->ntiles,
                                 cudaMemcpyHostToDevice, st));
        long *d_dst = nullptr;
        OSG_CUDA(cudaMalloc(&d_dst, sizeof(long) * np));
        OSG_CUDA(cudaMemcpyAsync(d_dst, dst.data(), sizeof(long) * np, cudaMemcpyHostToDevice, st));
        unsigned nb = blocks_for(np, 256);
        if (nb > 8192) nb = 8192;
        k_bin<<<nb, 256, 0, st>>>(dix, dx_, du, dq, d_dst, np, dim, t->buf[0][k]);
        cudaError_t ce = cudaStreamSynchronize(st);
        cudaFree(d_dst);
        OSG_CUDA(ce);
        OSG_CUDA(cudaGetLastError());
    } else {
        OSG_CUDA(cudaMemsetAsync(t->buf[0][k].cnt, 0, sizeof(int) * t->ntiles, st));
    }
    return upload_tables(t, st);
}

int tiled_push(TiledState *t, int parity, const float *e, const float *b, float *j,
               double *d_ene, int *d_status, cudaStream_t st, int *launches)
{
    const int ns = (int)t->rqm.size();
    if (ns == 0) return OSG_OK;
    // the push writes every tile's sorted count and adds arrivals to zeroed counters
    OSG_CUDA(cudaMemsetAsync(t->d_arr[1 - parity], 0, sizeof(int) * MAX_TILED_SPECIES * t->ntiles, st));
    TiledArgs a = base_args(t);
    a.e = e;
    a.b = b;
    a.j = j;
    a.spec = t->d_tab[parity];
    a.nspec = ns;
    a.ene = d_ene;
    a.status = d_status;
    a.reduce_min = t->reduce_min;
    const size_t sm = t->smem_bytes;
#define OSG_TCASE(D, O)                                                                       \
    if (t->dim == D && t->order == O) {                                                       \
        k_push_tiled<D, O><<<(unsigned)t->ntiles, t->threads, sm, st>>>(a);                          \
        *launches += 1;                                                                       \
        return OSG_OK;                                                                        \
    }
    OSG_TCASE(2, 1) OSG_TCASE(2, 2) OSG_TCASE(2, 3) OSG_TCASE(2, 4)
    OSG_TCASE(3, 1) OSG_TCASE(3, 2) OSG_TCASE(3, 3) OSG_TCASE(3, 4)
#undef OSG_TCASE
    set_error("tiled engine: unsupported dim %d order %d", t->dim, t->order);
    return OSG_ERR_ARG;
}

// particles per tile of species k in buffer `cur` (sorted part + arrivals, as the kernels read it)
static int tile_counts(TiledState *t, int cur, int k, std::vector<int> &n, cudaStream_t st)
{
    std::vector<int> c(t->ntiles), r(t->ntiles);
    OSG_CUDA(cudaMemcpyAsync(c.data(), t->buf[cur][k].cnt, sizeof(int) * t->ntiles,
                             cudaMemcpyDeviceToHost, st));
    OSG_CUDA(cudaMemcpyAsync(r.data(), t->buf[cur][k].arr, sizeof(int) * t->ntiles,
                             cudaMemcpyDeviceToHost, st));
    OSG_CUDA(cudaStreamSynchronize(st));
    n.resize(t->ntiles);
    const long cap = t->cap[k];
    for (long i = 0; i < t->ntiles; i++) {
        const long nst = std::min<long>(c[i], cap);
        n[i] = (int)(nst + std::min<long>(r[i], cap - nst));
    }
    return OSG_OK;
}

int tiled_count(TiledState *t, int cur, int k, long *np, cudaStream_t st)
{
    OSG_CHECK(k >= 0 && k < (int)t->rqm.size(), OSG_ERR_ARG, "bad species");
    std::vector<int> c;
    int rc = tile_counts(t, cur, k, c, st);
    if (rc) return rc;
    long n = 0;
    for (long i = 0; i < t->ntiles; i++) n += c[i];
    *np = n;
    return OSG_OK;
}

// compact species k of buffer `cur` into the reference layout in device scratch; returns count
static int compact(TiledState *t, int cur, int k, cudaStream_t st, long *np_out)
{
    std::vector<int> c, off(t->ntiles);
    int rc = tile_counts(t, cur, k, c, st);
    if (rc) return rc;
    long n = 0;
    for (long i = 0; i < t->ntiles; i++) {
        off[i] = (int)n;
        n += c[i];
    }
    const int dim = t->dim;
    const size_t need = (size_t)(n > 0 ? n : 1) * (sizeof(int) * dim + sizeof(float) * (dim + 4));
    if (need > t->compact_bytes) {
        cudaFree(t->d_compact);
        t->d_compact = nullptr;
        t->compact_bytes = 0;
        OSG_CUDA(cudaMalloc(&t->d_compact, need));
        t->compact_bytes = need;
    }
    OSG_CUDA(cudaMemcpyAsync(t->d_off, off.data(), sizeof(int) * t->ntiles, cudaMemcpyHostToDevice, st));
    int *dix = (int *)t->d_compact;
    float *dx_ = (float *)(dix + (size_t)dim * n);
    float *du = dx_ + (size_t)dim * n;
    float *dq = du + (size_t)3 * n;
    k_compact<<<(unsigned)t->ntiles, 128, 0, st>>>(t->buf[cur][k], t->cap[k], dim, t->d_off, dix,
                                                   dx_, du, dq);
    OSG_CUDA(cudaGetLastError());
    *np_out = n;
    return OSG_OK;
}

int tiled_get_species(TiledState *t, int cur, int k, int *ix, float *x, float *u, float *q,
                      cudaStream_t st)
{
    OSG_CHECK(k >= 0 && k < (int)t->rqm.size(), OSG_ERR_ARG, "bad species");
    long n;
    int rc = compact(t, cur, k, st, &n);
    if (rc) return rc;
    const int dim = t->dim;
    int *dix = (int *)t->d_compact;
    float *dx_ = (float *)(dix + (size_t)dim * n);
    float *du = dx_ + (size_t)dim * n;
    float *dq = du + (size_t)3 * n;
    if (n > 0) {
        if (ix) OSG_CUDA(cudaMemcpyAsync(ix, dix, sizeof(int) * dim * n, cudaMemcpyDeviceToHost, st));
        if (x) OSG_CUDA(cudaMemcpyAsync(x, dx_, sizeof(float) * dim * n, cudaMemcpyDeviceToHost, st));
        if (u) OSG_CUDA(cudaMemcpyAsync(u, du, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, st));
        if (q) OSG_CUDA(cudaMemcpyAsync(q, dq, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
    }
    OSG_CUDA(cudaStreamSynchronize(st));
    return OSG_OK;
}

int tiled_occupancy(TiledState *t, int cur, double *max_frac, cudaStream_t st)
{
    double m = 0.0;
    for (size_t k = 0; k < t->rqm.size(); k++) {
        std::vector<int> c;
        int rc = tile_counts(t, cur, (int)k, c, st);
        if (rc) return rc;
        for (long i = 0; i < t->ntiles; i++) m = std::max(m, (double)c[i] / (double)t->cap[k]);
    }
    *max_frac = m;
    return OSG_OK;
}

// Re-bin every species into slabs sized for the current particle distribution (host round
// trip: compact -> host -> sorted re-bin).  Used between step batches when a tile fills up.
int tiled_regrow(TiledState *t, int cur, cudaStream_t st)
{
    const int ns = (int)t->rqm.size();
    const int dim = t->dim;
    std::vector<std::vector<int>> ix(ns);
    std::vector<std::vector<float>> x(ns), u(ns), q(ns);
    for (int k = 0; k < ns; k++) {
        long n = 0;
        int rc = tiled_count(t, cur, k, &n, st);
        if (rc) return rc;
        ix[k].resize((size_t)dim * n);
        x[k].resize((size_t)dim * n);
        u[k].resize((size_t)3 * n);
        q[k].resize((size_t)n);
        rc = tiled_get_species(t, cur, k, ix[k].data(), x[k].data(), u[k].data(), q[k].data(), st);
        if (rc) return rc;
    }
    std::vector<double> rqm = t->rqm;
    for (void *p : t->allocs) cudaFree(p);
    t->allocs.clear();
    t->buf[0].clear();
    t->buf[1].clear();
    t->rqm.clear();
    t->cap.clear();
    for (int p = 0; p < 2; p++) {
        OSG_CUDA(cudaMemsetAsync(t->d_cnt[p], 0, sizeof(int) * MAX_TILED_SPECIES * t->ntiles, st));
        OSG_CUDA(cudaMemsetAsync(t->d_arr[p], 0, sizeof(int) * MAX_TILED_SPECIES * t->ntiles, st));
    }
    for (int k = 0; k < ns; k++) {
        const long n = (long)q[k].size();
        int rc = tiled_add_species(t, rqm[k], n, ix[k].data(), x[k].data(), u[k].data(),
                                   q[k].data(), st);
        if (rc) return rc;
    }
    if (cur == 1) {
        // the particles were binned into buffer 0; the caller's next step reads buffer `cur`
        for (int k = 0; k < ns; k++) std::swap(t->buf[0][k], t->buf[1][k]);
        std::swap(t->d_cnt[0], t->d_cnt[1]);
        std::swap(t->d_arr[0], t->d_arr[1]);
        for (int k = 0; k < ns; k++) {
            for (int p = 0; p < 2; p++) {
                t->buf[p][k].cnt = t->d_cnt[p] + (size_t)k * t->ntiles;
                t->buf[p][k].arr = t->d_arr[p] + (size_t)k * t->ntiles;
            }
        }
        return upload_tables(t, st);
    }
    return OSG_OK;
}

int tiled_deposit_rho(TiledState *t, int cur, int k, double *rho, int *status, cudaStream_t st)
{
    long n;
    int rc = compact(t, cur, k, st, &n);
    if (rc) return rc;
    const int dim = t->dim;
    int *dix = (int *)t->d_compact;
    float *dx_ = (float *)(dix + (size_t)dim * n);
    float *du = dx_ + (size_t)dim * n;
    float *dq = du + (size_t)3 * n;
    return deposit_rho<float>(t->g, t->order, dix, dx_, dq, n, rho, status, st);
}

} // namespace osg
