// tiled.cu -- single-precision particle engine with particles binned by spatial tile.
//
// Layout in HBM: for every species two particle buffers (ping-pong), each a set of SoA
// streams (cell index per axis, in-cell offset per axis, three momenta, charge) cut into
// fixed-capacity slabs, one slab per tile; a per-tile count says how many slots are live.
//
// One push launch handles every species: CTA t owns tile t.  It stages E and B of the tile
// plus the stencil halo in shared memory, zeroes a shared-memory current tile with its halo,
// and for each species streams the tile's particles (coalesced SoA loads), gathers the fields
// from shared memory, does the Boris push, moves, trims and periodically wraps the particle,
// splits the trajectory at cell faces and accumulates the charge-conserving current of every
// segment into the shared tile (shared-memory atomics), then writes the particle into the
// slab of the tile that now contains it in the other buffer (warp-aggregated slot reservation
// for particles that stay, one atomic per particle that leaves).  The shared current tile is
// added to the global current at the end (the halo overlaps the neighbours' halos).
//
// The per-particle arithmetic is the same as the plain engine (pic_math.cuh) and therefore the
// same as the reference kernels FNAME(vadvance_deposit_{2d,3d}_sN) (source/simd/
// os-spec-push-avx2.c:471-760, :1141-1480); only the order in which current contributions are
// summed differs.  The particle migration replaces both the periodic particle boundary
// (source/spec/os-spec-boundary.f03:1280-1290) and the cell sort (source/spec/os-species.f03:
// 269-505): particles are re-binned by tile every step.
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
    int *cnt;      // [ntiles]
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
    int local_sort;    // write stayers of each block iteration in cell order
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
    int *d_off = nullptr;
    void *d_compact = nullptr;
    size_t compact_bytes = 0;
    size_t smem_bytes = 0;
    int threads = 128;   // threads per push CTA (multiple of 32, <= 256)
    int local_sort = 1;
    int reduce_min = 2;
};

static const int MAX_TILED_SPECIES = 16;
static const int MAX_TILE_CELLS = 1024;   // cells per tile (shared counting-sort bins)

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
template <int DIM, int ORD>
__global__ void __launch_bounds__(256) k_push_tiled(TiledArgs a)
{
    constexpr int NP = ORD + 1, OFS = Stencil<ORD>::OFS;
    constexpr int MAXSEG = DIM == 2 ? 3 : 4;
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
    float *sE = smem, *sB = smem + 3 * ne, *sJ = smem + 6 * ne;
    const long gsy = 3L * a.size[0], gsz = 3L * a.size[0] * a.size[1];

    // stage fields: local point l <-> Fortran cell t0 - OFS + l <-> global position
    // t0 - OFS + l - 1 + gcl (inside the guard cells for tiles at the box edge)
    for (int idx = threadIdx.x; idx < 3 * ne; idx += blockDim.x) {
        const int c = idx % 3, pnt = idx / 3;
        const int lx = pnt % ee[0], ly = (pnt / ee[0]) % ee[1], lz = pnt / (ee[0] * ee[1]);
        long gp = 3L * (t0[0] - OFS + lx - 1 + a.gcl[0]) + c;
        if (DIM > 1) gp += gsy * (t0[1] - OFS + ly - 1 + a.gcl[1]);
        if (DIM > 2) gp += gsz * (t0[2] - OFS + lz - 1 + a.gcl[2]);
        sE[idx] = __ldg(a.e + gp);
        sB[idx] = __ldg(a.b + gp);
    }
    for (int idx = threadIdx.x; idx < 3 * nj; idx += blockDim.x) sJ[idx] = 0.0f;
    __syncthreads();

    const int esy = 3 * ee[0], esz = 3 * ee[0] * ee[1];
    const int jsy = 3 * je[0], jsz = 3 * je[0] * je[1];
    const unsigned lane = threadIdx.x & 31;

    // segment buffer: [0, blockDim) first segment of each thread's particle (particle order),
    // [blockDim, MAXSEG * blockDim) the extra segments of split trajectories, compacted
    SegRec *sSeg = reinterpret_cast<SegRec *>(smem + ((6 * ne + 3 * nj + 3) & ~3));
    // per-iteration counters, double-buffered so the spare copy is cleared while the other is
    // in use (three block barriers per iteration)
    __shared__ int sNextra[2], sStayBase;
    __shared__ int sCellCnt[2][MAX_TILE_CELLS];
    const int nthr = blockDim.x;
    const int ncell_tile = a.T[0] * a.T[1] * a.T[2];
    for (int k = threadIdx.x; k < ncell_tile; k += nthr) sCellCnt[0][k] = sCellCnt[1][k] = 0;
    if (threadIdx.x == 0) sNextra[0] = sNextra[1] = 0;
    __syncthreads();
    int it = 0;

    for (int s = 0; s < a.nspec; s++) {
        const SpeciesDev sd = a.spec[s];
        const long cap = sd.cap;
        const long slab = tile * cap;
        int cnt = sd.in.cnt[tile];
        if (cnt > cap) cnt = (int)cap;
        // per-thread partial energy in FP32 (the reference sums in single precision per
        // 464-particle chunk), summed over the block in double
        float my_ene = 0.f;
        for (int base = 0; base < cnt; base += nthr, it++) {
            const int bp = it & 1;
            int *cellCnt = sCellCnt[bp];
            const int i = base + threadIdx.x;
            bool has = i < cnt;
            int c[3] = {1, 1, 1}, cw[3] = {1, 1, 1}, di[3] = {0, 0, 0};
            float xo[3] = {0, 0, 0}, x1[3] = {0, 0, 0}, un[3] = {0, 0, 0}, q = 0.0f;
            if (has) {
                const long p = slab + i;
                bool ok = true;
#pragma unroll
                for (int d = 0; d < DIM; d++) {
                    c[d] = sd.in.ix[d][p];
                    xo[d] = sd.in.x[d][p];
                    const int lc = c[d] - t0[d];
                    ok = ok && lc >= 0 && lc < a.T[d];
                }
                un[0] = sd.in.u[0][p];
                un[1] = sd.in.u[1][p];
                un[2] = sd.in.u[2][p];
                q = sd.in.q[p];
                if (!ok) {
                    atomicOr(a.status, OSG_STATUS_RANGE);
                    has = false;
                }
            }
            // ---- phase 1: gather from the staged tile, Boris, move, split into segments
            int nseg = 0;
            SegRec sg[MAXSEG];
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
            // primary segment in particle order, extras compacted after the primaries
            sSeg[threadIdx.x] = sg[0];
            if (!has) sSeg[threadIdx.x].base = -1;
            {
                const int nx_ = has ? nseg - 1 : 0;
                int incl = nx_;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(FULL_MASK, incl, o);
                    if ((int)lane >= o) incl += y;
                }
                const int wtot = __shfl_sync(FULL_MASK, incl, 31);
                int wbase = 0;
                if (lane == 31 && wtot) wbase = atomicAdd(&sNextra[bp], wtot);
                wbase = __shfl_sync(FULL_MASK, wbase, 31);
                int o = nthr + wbase + incl - nx_;
                for (int t = 1; t < nseg; t++) sSeg[o++] = sg[t];
            }
            // ---- new position, cell (periodically wrapped) and destination tile
            long dest = -1;
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
            // ---- migration.  Particles that stay are written in cell order (block counting
            //      sort over the tile's cells) so that next step the lanes of a warp mostly share
            //      a cell; particles that leave take one slot each in their destination tile.
            const bool stay = has && dest == tile;
            long slot = -1;
            if (a.local_sort) {
                int lcell = 0, rank = 0;
                if (stay) {
                    lcell = cw[0] - t0[0];
                    if (DIM > 1) lcell += a.T[0] * (cw[1] - t0[1]);
                    if (DIM > 2) lcell += a.T[0] * a.T[1] * (cw[2] - t0[2]);
                    rank = atomicAdd(&cellCnt[lcell], 1);
                }
                __syncthreads();
                if (threadIdx.x < 32) {
                    const int nstay = warp_exclusive_scan(cellCnt, ncell_tile);
                    if (threadIdx.x == 0) sStayBase = nstay ? atomicAdd(sd.out.cnt + tile, nstay) : 0;
                }
                __syncthreads();
                if (stay) slot = sStayBase + cellCnt[lcell] + rank;
            } else {
                // warp-aggregated slots in the own tile, particle order kept per warp
                const unsigned ms = __ballot_sync(FULL_MASK, stay);
                if (ms) {
                    const int leader = __ffs(ms) - 1;
                    int b0 = 0;
                    if ((int)lane == leader) b0 = atomicAdd(sd.out.cnt + tile, __popc(ms));
                    b0 = __shfl_sync(FULL_MASK, b0, leader);
                    if (stay) slot = b0 + __popc(ms & ((1u << lane) - 1u));
                }
            }
            if (has && !stay) slot = atomicAdd(sd.out.cnt + dest, 1);
            if (has) {
                if (slot >= cap) {
                    atomicOr(a.status, OSG_STATUS_OVERFLOW);
                } else {
                    const long o = dest * cap + slot;
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
            }
            if (!a.local_sort) __syncthreads();   // segment buffer complete
            // clear the spare counters for the next iteration
            int *spare = sCellCnt[bp ^ 1];
            for (int k = threadIdx.x; k < ncell_tile; k += nthr) spare[k] = 0;
            if (threadIdx.x == 0) sNextra[bp ^ 1] = 0;
            // ---- phase 2: charge-conserving current of all segments into the shared tile
            const int nall = nthr + sNextra[bp];
            for (int r = 0; r * nthr < nall; r++) {
                int sidx = r * nthr + threadIdx.x;
                if (DIM == 3 && r == 0 && (direct_only<DIM, ORD>() || a.reduce_min > 32)) sidx = spread_index(threadIdx.x, nthr);
                const bool valid = sidx < nall && sSeg[sidx].base >= 0;
                deposit_segment<DIM, ORD>(sJ, valid ? &sSeg[sidx] : nullptr, a.jn, jsy, jsz,
                                          a.reduce_min);
            }
            __syncthreads();
        }
        const double tot = block_sum((double)my_ene);
        if (threadIdx.x == 0 && tot != 0.0) atomicAdd(a.ene + s, tot);
    }
    __syncthreads();
    // ---- add the shared current tile (with halo) to the global current
    for (int idx = threadIdx.x; idx < 3 * nj; idx += blockDim.x) {
        const float v = sJ[idx];
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

// --------------------------------------------------------------------------------- sort
// Full counting sort of every tile by cell (x fastest inside the tile): reads the slabs of
// spec[s].in, writes spec[s].out.  The GPU counterpart of the reference's cell sort every
// n_sort steps (source/spec/os-species.f03:269-505), per tile instead of over the whole box.
__global__ void __launch_bounds__(256) k_tile_sort(TiledArgs a, int dim)
{
    extern __shared__ int hist[];
    const long tile = blockIdx.x;
    const SpeciesDev sd = a.spec[blockIdx.y];
    const long cap = sd.cap;
    int n = sd.in.cnt[tile];
    if (n > cap) n = (int)cap;
    const int ncell = a.T[0] * a.T[1] * a.T[2];
    int t0[3];
    {
        long r = tile;
        for (int d = 0; d < 3; d++) {
            t0[d] = (int)(r % a.ntile[d]) * a.T[d] + 1;
            r /= a.ntile[d];
        }
    }
    for (int k = threadIdx.x; k < ncell; k += blockDim.x) hist[k] = 0;
    __syncthreads();
    const long base = tile * cap;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        int lc = sd.in.ix[0][base + i] - t0[0];
        if (dim > 1) lc += a.T[0] * (sd.in.ix[1][base + i] - t0[1]);
        if (dim > 2) lc += a.T[0] * a.T[1] * (sd.in.ix[2][base + i] - t0[2]);
        atomicAdd(&hist[min(max(lc, 0), ncell - 1)], 1);
    }
    __syncthreads();
    if (threadIdx.x < 32) warp_exclusive_scan(hist, ncell);
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const long src = base + i;
        int lc = sd.in.ix[0][src] - t0[0];
        if (dim > 1) lc += a.T[0] * (sd.in.ix[1][src] - t0[1]);
        if (dim > 2) lc += a.T[0] * a.T[1] * (sd.in.ix[2][src] - t0[2]);
        const long dst = base + atomicAdd(&hist[min(max(lc, 0), ncell - 1)], 1);
        for (int d = 0; d < dim; d++) {
            sd.out.ix[d][dst] = sd.in.ix[d][src];
            sd.out.x[d][dst] = sd.in.x[d][src];
        }
        sd.out.u[0][dst] = sd.in.u[0][src];
        sd.out.u[1][dst] = sd.in.u[1][src];
        sd.out.u[2][dst] = sd.in.u[2][src];
        sd.out.q[dst] = sd.in.q[src];
    }
    if (threadIdx.x == 0) sd.out.cnt[tile] = n;
}

// slab -> reference layout (ix(dim,N), x(dim,N), p(3,N), q(N)) at offsets off[tile]
__global__ void k_compact(Slabs in, long cap, int dim, const int *__restrict__ off, int *ix,
                          float *x, float *u, float *q)
{
    const long t = blockIdx.x;
    int n = in.cnt[t];
    if (n > cap) n = (int)cap;
    const long o = off[t];
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const long src = t * cap + i, dst = o + i;
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

// shared memory of the push kernel: E and B tiles, the current tile, the segment buffer
static size_t smem_for(int dim, int order, const int *T, int threads)
{
    const int NP = order + 1;
    size_t ne = 1, nj = 1;
    for (int d = 0; d < dim; d++) {
        ne *= (size_t)(T[d] + NP);
        nj *= (size_t)(T[d] + NP + 1);
    }
    const size_t fields = ((6 * ne + 3 * nj + 3) & ~(size_t)3) * sizeof(float);
    return fields + sizeof(SegRec) * (dim == 2 ? 3 : 4) * threads;
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
    if ((long)t->T[0] * t->T[1] * t->T[2] > MAX_TILE_CELLS) {
        set_error("a tile may hold at most %d cells", MAX_TILE_CELLS);
        delete t;
        return OSG_ERR_ARG;
    }
    if (const char *ev = getenv("OSG_LOCAL_SORT")) t->local_sort = atoi(ev) != 0;
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
            cudaMalloc(&t->d_tab[p], sizeof(SpeciesDev) * MAX_TILED_SPECIES) != cudaSuccess) {
            tiled_destroy(t);
            set_error("tile count allocation failed");
            return OSG_ERR_NOMEM;
        }
        cudaMemset(t->d_cnt[p], 0, sizeof(int) * MAX_TILED_SPECIES * t->ntiles);
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
    OSG_CUDA(cudaMemsetAsync(t->d_cnt[1 - parity], 0, sizeof(int) * MAX_TILED_SPECIES * t->ntiles, st));
    TiledArgs a = base_args(t);
    a.e = e;
    a.b = b;
    a.j = j;
    a.spec = t->d_tab[parity];
    a.nspec = ns;
    a.ene = d_ene;
    a.status = d_status;
    a.local_sort = t->local_sort;
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

int tiled_sort(TiledState *t, int in_buf, cudaStream_t st, int *launches)
{
    const int ns = (int)t->rqm.size();
    if (ns == 0) return OSG_OK;
    TiledArgs a = base_args(t);
    a.spec = t->d_tab[in_buf];
    a.nspec = ns;
    const int ncell = t->T[0] * t->T[1] * t->T[2];
    dim3 grid((unsigned)t->ntiles, (unsigned)ns);
    k_tile_sort<<<grid, 256, sizeof(int) * ncell, st>>>(a, t->dim);
    *launches += 1;
    return OSG_OK;
}

int tiled_count(TiledState *t, int cur, int k, long *np, cudaStream_t st)
{
    OSG_CHECK(k >= 0 && k < (int)t->rqm.size(), OSG_ERR_ARG, "bad species");
    std::vector<int> c(t->ntiles);
    OSG_CUDA(cudaMemcpyAsync(c.data(), t->buf[cur][k].cnt, sizeof(int) * t->ntiles,
                             cudaMemcpyDeviceToHost, st));
    OSG_CUDA(cudaStreamSynchronize(st));
    long n = 0;
    for (long i = 0; i < t->ntiles; i++) n += std::min<long>(c[i], t->cap[k]);
    *np = n;
    return OSG_OK;
}

// compact species k of buffer `cur` into the reference layout in device scratch; returns count
static int compact(TiledState *t, int cur, int k, cudaStream_t st, long *np_out)
{
    std::vector<int> c(t->ntiles), off(t->ntiles);
    OSG_CUDA(cudaMemcpyAsync(c.data(), t->buf[cur][k].cnt, sizeof(int) * t->ntiles,
                             cudaMemcpyDeviceToHost, st));
    OSG_CUDA(cudaStreamSynchronize(st));
    long n = 0;
    for (long i = 0; i < t->ntiles; i++) {
        off[i] = (int)n;
        n += std::min<long>(c[i], t->cap[k]);
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
    std::vector<int> c(t->ntiles);
    for (size_t k = 0; k < t->rqm.size(); k++) {
        OSG_CUDA(cudaMemcpyAsync(c.data(), t->buf[cur][k].cnt, sizeof(int) * t->ntiles,
                                 cudaMemcpyDeviceToHost, st));
        OSG_CUDA(cudaStreamSynchronize(st));
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
    for (int p = 0; p < 2; p++)
        OSG_CUDA(cudaMemsetAsync(t->d_cnt[p], 0, sizeof(int) * MAX_TILED_SPECIES * t->ntiles, st));
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
        for (int k = 0; k < ns; k++) {
            t->buf[0][k].cnt = t->d_cnt[0] + (size_t)k * t->ntiles;
            t->buf[1][k].cnt = t->d_cnt[1] + (size_t)k * t->ntiles;
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
