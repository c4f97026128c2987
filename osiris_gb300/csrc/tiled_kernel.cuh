// tiled_kernel.cuh -- device side of the tiled particle engine: slab layout, launch arguments
// and the push + deposit + migration kernel k_push_tiled<DIM, ORD, PUSHER>.  Included by
// tiled.cu (Boris instantiations, host code) and tiled_exact.cu (exact-pusher instantiations),
// so the two sets compile in parallel.
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"
#include "pic_math.cuh"
#include "push_plain.cuh"
#include "tile_ops.cuh"

namespace osg {

// Particle records of the tiled engine, one per slot: 2D {ix1, ix2, x1, x2, u1, u2, u3, q}
// (32 bytes), 3D {ix1, ix2, ix3, x1, x2, x3, u1, u2, u3, q, 0, 0} (48 bytes); the cell indices
// are stored as int bits.  A 2D record moves as one 32-byte vector access (sm_100+
// ld/st.global.v8: a warp's 32 records are 1 KB of whole lines, one instruction), a 3D record
// as three 16-byte vectors.
template <int DIM> struct PRec {
    static constexpr int N = DIM == 2 ? 8 : 12;   // floats per record
};

struct Slabs {
    float *rec;    // records, slot i of tile t at t * cap + i
    int *cnt;      // [ntiles] particles in slots [0, cnt) of the slab, sorted by cell
    int *arr;      // [ntiles] particles that arrived from other tiles, slots [cap - arr, cap)
};

template <int DIM>
__device__ __forceinline__ void load_rec(const float *rec, long p, int *c, float *x, float *u,
                                         float &q)
{
    const float4 *r = reinterpret_cast<const float4 *>(rec + p * PRec<DIM>::N);
    if constexpr (DIM == 2) {
        float c0, c1;
        asm volatile("ld.global.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                     : "=f"(c0), "=f"(c1), "=f"(x[0]), "=f"(x[1]), "=f"(u[0]), "=f"(u[1]),
                       "=f"(u[2]), "=f"(q)
                     : "l"(r)
                     : "memory");
        c[0] = __float_as_int(c0);
        c[1] = __float_as_int(c1);
    } else {
        const float4 a = r[0], b = r[1], d = r[2];
        c[0] = __float_as_int(a.x);
        c[1] = __float_as_int(a.y);
        c[2] = __float_as_int(a.z);
        x[0] = a.w;
        x[1] = b.x;
        x[2] = b.y;
        u[0] = b.z;
        u[1] = b.w;
        u[2] = d.x;
        q = d.y;
    }
}

// STREAM: a record of the output buffer, not read again in this step -- stored with the
// evict-first policy (.cs), so that it does not push out of L2 the input-slab lines that the
// sort pass still has to read
template <int DIM, bool STREAM = false>
__device__ __forceinline__ void store_rec(float *rec, long p, const int *c, const float *x,
                                          const float *u, float q)
{
    float4 *r = reinterpret_cast<float4 *>(rec + p * PRec<DIM>::N);
    if constexpr (DIM == 2) {
        if constexpr (STREAM)
            asm volatile("st.global.cs.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(r),
                         "f"(__int_as_float(c[0])), "f"(__int_as_float(c[1])), "f"(x[0]),
                         "f"(x[1]), "f"(u[0]), "f"(u[1]), "f"(u[2]), "f"(q)
                         : "memory");
        else
            asm volatile("st.global.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(r),
                         "f"(__int_as_float(c[0])), "f"(__int_as_float(c[1])), "f"(x[0]),
                         "f"(x[1]), "f"(u[0]), "f"(u[1]), "f"(u[2]), "f"(q)
                         : "memory");
    } else {
        const float4 r0 = make_float4(__int_as_float(c[0]), __int_as_float(c[1]),
                                      __int_as_float(c[2]), x[0]);
        const float4 r1 = make_float4(x[1], x[2], u[0], u[1]);
        const float4 r2 = make_float4(u[2], q, 0.f, 0.f);
        if constexpr (STREAM) {
            __stcs(r, r0);
            __stcs(r + 1, r1);
            __stcs(r + 2, r2);
        } else {
            r[0] = r0;
            r[1] = r1;
            r[2] = r2;
        }
    }
}

// first cell index of a record (0 marks an empty slot)
template <int DIM>
__device__ __forceinline__ int *rec_ix0(float *rec, long p)
{
    return reinterpret_cast<int *>(rec + p * PRec<DIM>::N);
}

struct SpeciesDev {
    Slabs in, out;
    float tem;     // dt / (2 rqm) (Boris)
    float qm;      // 1 / rqm (exact pusher)
    float rqm;     // rqm (Euler-rotation pusher)
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
    double dt_full;    // exact pusher: the double time step and the Newton tolerance
    double iter_tol;
    // current of every tile with its halo, [tile][3 * points] (hi) and its compensation (lo),
    // summed in FP64 in tile order by k_tile_fold
    float *tile_hi;
    float *tile_lo;
    // per tile: 1 when it held no particle of any species this step (its current buffer is
    // then not written, and the fold skips it), else 0
    int *tile_empty;
    // 3D: the tile current is accumulated as fixed point, value x 2^S split into a low word
    // of B bits and a high word (fx.scale = 2^S, fx.shift = B; chosen so that no tile point,
    // nor the fold's sum of tiles, can overflow)
    FxFormat fx;
    // bit d: axis d is not periodic and absorbs particles at both edges (the axis of Lindman
    // open boundaries).  window = 1: x1 is the moving window's axis (absorbing below,
    // reflecting above), and shift_x = 1 (a step that ends with a window move) stores every
    // particle one cell lower in x1
    int open;
    int window;
    int shift_x;
    // bit d: axis d is bounded by conducting walls (particles reflect specularly)
    int walls;
    // bit d (a walled or open axis): particles crossing its edges are re-emitted from a thermal
    // bath (tiled_reemit): distribution thermal_type, momenta uth_bnd / ufl_bnd, random stream
    // keyed by (seed, species) with the step counter at *step
    int thermal;
    int thermal_type;
    unsigned int seed;
    const unsigned long long *step;
    float uth_bnd[3];
    float ufl_bnd[3];
    // 1: drop the dead input-slab lines from L2 after the sort (discard_dead_slab).  0 for
    // multi-pass profiler replay, which saves and restores memory and needs it defined
    int discard;
};

// words of padding per row and per plane of the 3D current tile (bank spread of the lanes'
// fixed-point adds): none -- with the deposit's (plane, index) lane rotation, one or five words
// per row (and 16 per plane) measured 0-4% slower on configurations 3 and 5
__host__ __device__ constexpr int j3_pad_y(int) { return 0; }
__host__ __device__ constexpr int j3_pad_z(int) { return 0; }

static const int MAX_TILED_SPECIES = 16;
static const int MAX_TILE_CELLS = 1024;   // cells per tile (bins of the per-tile cell sort)
// the sort key a stayer carries between the two passes: 1 + cell in the tile + rank << bits
static const int SORT_CELL_BITS = 10;
static const long MAX_TILE_SLOTS = (1L << (31 - SORT_CELL_BITS)) - 1;   // ranks that fit

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
static const int LEAVE_QUEUE = 128;   // particles per CTA and species queued for emigration

// Write a particle that left its tile into an arrival slot (from the top of the slab) of its
// destination tile in the output buffer.  The arrival region stays above the particles the
// destination keeps this step: those are at most its input particles.
template <int DIM>
__device__ __forceinline__ void emigrate(const SpeciesDev &sd, long cap, long dest,
                                         const int *cw, const float *xo, const float *un,
                                         float q, int *status)
{
    // (the destination's input counts are loaded before the atomic: one round trip for both)
    const int room = (int)cap - sd.in.cnt[dest] - sd.in.arr[dest];
    const int k = atomicAdd(sd.out.arr + dest, 1);
    if (k >= room) {
        atomicOr(status, OSG_STATUS_OVERFLOW);
        return;
    }
    store_rec<DIM, true>(sd.out.rec, dest * cap + cap - 1 - k, cw, xo, un, q);
}

// After the sort, a tile's input slab is dead until the next step writes it as its output:
// the cache lines the first pass dirtied (stayers written back to their own slots, [0, nst)
// and the arrival region [cap - nar, cap)) are dropped from L2 without a write-back to DRAM.
// A tile's slab starts on a 128-byte line and spans whole lines (cap is a multiple of 32
// slots of 32 or 48 bytes, the allocation 128-byte aligned).
template <int DIM>
__device__ __forceinline__ void discard_dead_slab(const Slabs &in, long slab, int nst, int nar,
                                                  long cap)
{
    constexpr int RB = 4 * PRec<DIM>::N;   // bytes per record
    const int lo_lines = (nst * RB + 127) >> 7;
    const int cap_lines = (int)((cap * RB) >> 7);
    const int hi_first = max((int)(((cap - nar) * RB) >> 7), lo_lines);
    const int nl = lo_lines + (nar > 0 ? cap_lines - hi_first : 0);
    const char *base = reinterpret_cast<const char *>(in.rec + slab * PRec<DIM>::N);
    for (int l0 = threadIdx.x; l0 < nl; l0 += blockDim.x) {
        const int line = l0 < lo_lines ? l0 : hi_first + (l0 - lo_lines);
        const char *pa = base + 128L * line;
        asm volatile("discard.global.L2 [%0], 128;" ::"l"(pa) : "memory");
    }
}

// Every warp of the CTA runs its own pipeline over chunks of 32 particles of the tile, with no
// block barrier inside the particle loop: load, gather, Boris, move, split, write the particle
// to its new slot, then deposit the segments (round t takes the t-th segment of every lane).
// In 2D every warp accumulates into its own copy of the current tile (with a two-sum
// compensation), so its adds are plain shared read-modify-writes; the copies are summed when
// the tile is flushed.  In 3D the warps share one current tile, accumulated exactly as fixed
// point by 32-bit integer atomics (lanes_deposit3).
// CTAs of up to 256 threads.  2D linear/quadratic: three resident CTAs per SM (at most 85
// registers per thread, measured fastest on GB300); 2D quartic: one (it needs ~250 registers
// without spilling); otherwise two
template <int DIM, int ORD>
constexpr int push_min_blocks() { return DIM == 2 ? (ORD <= 2 ? 3 : (ORD == 3 ? 2 : 1)) : 2; }

// Thermal-bath re-emission in the tiled engine (p_bc_thermal, source/spec/os-spec-boundary.f03:
// 1315-1387, thermal_bath :972-1067, rev_current :1392-1440), for a particle whose move
// crossed the bath edges coded in tb (2 bits per axis: 1 lower, 2 upper), axis by axis as the
// plain engine's thermal_reemit: the cell along d becomes the edge cell, the momenta come from
// bath_draw, the offset along d is xpos + u_d / gamma dt/dx_d v (xpos = -1/2 or the float just
// below 1/2), and the current of the way in, -q from the new position back along
// -u / gamma dt/dx, goes into the tile: in 2D by FP32 atomics into the warp's copy, in 3D by
// the exact fixed-point adds.  cn: the cells after the move before any wrap (the path's start
// cell in the tile's frame); cw receives the cells the particle is stored at.  The random
// stream is keyed by (seed, species) with the counter (id, step, axis and side); id, the
// particle's input slot, is unique within a species and step.  Particles of the tiled engine
// have no fixed index, so the stream is not the plain engine's: the same distributions.
template <int DIM, int ORD>
__device__ __noinline__ void tiled_reemit(const TiledArgs &a, int s, long id, int tb,
                                          const int *t0, const int *cn, int *cw, float *xo,
                                          float *un, float q, float *sJw, unsigned *sJl,
                                          unsigned *sJh, int jsy, int jsz)
{
    int lc[3] = {0, 0, 0};
    for (int k = 0; k < DIM; k++) lc[k] = cn[k];
    for (int d = 0; d < DIM; d++) {
        const int code = (tb >> (2 * d)) & 3;
        if (!code) continue;
        const bool lower = code == 1;
        cw[d] = lower ? 1 : a.nx[d];
        lc[d] = cw[d];
        double v3;
        bath_draw<float>(a.uth_bnd, a.ufl_bnd, a.thermal_type, d, lower, (unsigned long long)id,
                         (unsigned int)*a.step, a.seed, (unsigned int)s, un, &v3);
        const float rg = 1.0f / sqrtf(1.0f + un[0] * un[0] + un[1] * un[1] + un[2] * un[2]);
        const float xpos = lower ? -0.5f : 0.49999997f;
        const float vperp = rg * un[d] * a.dtdx[d];
        xo[d] = xpos + vperp * (float)v3;
        float xv[3] = {0.f, 0.f, 0.f};
        int di[3] = {0, 0, 0};
        for (int k = 0; k < DIM; k++) {
            xv[k] = xo[k] - un[k] * rg * a.dtdx[k];
            di[k] = trim(xv[k]);
        }
        SegRec sg[DIM == 2 ? 3 : 4];
        const int ns = make_segments<DIM>(sg, xo, xv, di, un[2] * rg, -q, lc[0] - t0[0] + 1,
                                          DIM > 1 ? lc[1] - t0[1] + 1 : 0,
                                          DIM > 2 ? lc[2] - t0[2] + 1 : 0, jsy, jsz);
        for (int t = 0; t < ns; t++) {
            if constexpr (DIM == 2) {
                constexpr int NV = SegVals<2, ORD>::NV;
                float v[NV];
                seg_values2_fast<ORD>(seg2_of<ORD>(sg[t]), sg[t].q, a.jn[0], a.jn[1], v);
                for (int k = 0; k < NV; k++)
                    atomicAdd(sJw + sg[t].base + seg_offset<2, ORD>(k, jsy, 0), v[k]);
            } else {
                lanes_deposit3<ORD>(sJl, sJh, sg[t], true, a.jn, jsy, jsz, a.fx);
            }
        }
    }
}

// The whole push of one tile by the calling CTA (all threads; contains block barriers; a CTA
// that pushes several tiles in a row puts a block barrier between the calls).
// DYN: the warps take the tile's 32-particle chunks from a shared counter (less waiting at the
// block barrier behind the slowest warp: 1.7% faster on the two-stream workload); otherwise
// warp w takes chunks w, w + warps, ... (the persistent batch, whose light tiles are one chunk
// per warp: 2.9% faster there)
// BATH: the thermal-bath particle boundary is compiled in (a variant of its own: its code in
// the push loop cost the other kernels 14-43% through register allocation)
template <int DIM, int ORD, int PUSHER, bool DYN, bool BATH>
__device__ __forceinline__ void push_tile(const TiledArgs &a, const long tile)
{
    constexpr int NP = ORD + 1, OFS = Stencil<ORD>::OFS;
    constexpr int MAXSEG = DIM == 2 ? 3 : 4;
    extern __shared__ float smem[];
    // a tile without particles (the vacuum of a sparse box) has nothing to push or deposit:
    // its output counts are 0 and the fold skips its current buffer
    {
        __shared__ int sAny;
        if (threadIdx.x == 0) {
            int any = 0;
            for (int s = 0; s < a.nspec; s++) {
                const SpeciesDev &sd = a.spec[s];
                any |= sd.in.cnt[tile] | sd.in.arr[tile];
            }
            sAny = any;
            a.tile_empty[tile] = any ? 0 : 1;
            if (!any)
                for (int s = 0; s < a.nspec; s++) a.spec[s].out.cnt[tile] = 0;
        }
        __syncthreads();
        const bool empty = sAny == 0;
        __syncthreads();   // sAny is read by every thread before a next tile of the CTA
        if (empty) return;
    }
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
    // current tile strides ([z][y][x][3], 3D rows and planes padded)
    const int jsy = 3 * je[0] + (DIM == 3 ? j3_pad_y(ORD) : 0);
    const int jsz = jsy * je[1] + (DIM == 3 ? j3_pad_z(ORD) : 0);
    const int njall = DIM == 2 ? 3 * nj * nwarp : jsz * je[2];
    // 2D: the warp copies of the current tile keep a two-sum compensation at offset jlo;
    // 3D: the low (offset 0) and high (offset jlo) words of the fixed-point tile current
    const int jlo = njall;
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
    for (int idx = threadIdx.x; idx < njall + jlo; idx += nthr) sJ[idx] = 0.0f;
    unsigned *sJl = reinterpret_cast<unsigned *>(sJ), *sJh = sJl + jlo;
    // dynamic shared memory after the current tile (16-byte aligned): per-warp value scratch
    // (2D) and queue of face-crossing segments, then two per-cell histograms of the tile sort (one
    // per species, alternating, so the next one is cleared while the current one is used)
    constexpr int SCRF = DIM == 2 ? scratch_floats2<ORD>() : 0;
    constexpr int QCAP = DIM == 2 ? SEGQ : SEGQ3;
    float *scr = smem + ((6 * ne + njall + jlo + 3) & ~3);
    SegRec *sQ0 = reinterpret_cast<SegRec *>(scr + nwarp * SCRF);
    int *sHist = reinterpret_cast<int *>(sQ0 + nwarp * QCAP);
    const int ncell = a.T[0] * a.T[1] * a.T[2];
    for (int k = threadIdx.x; k < ncell; k += nthr) sHist[k] = 0;
    // particles leaving the tile wait in a shared queue; after the pass they take their
    // arrival slots all at once, so no warp waits on a global atomic inside the pass
    __shared__ int sLeaveI[LEAVE_QUEUE][4];      // new cell per axis, destination tile
    __shared__ float sLeaveF[LEAVE_QUEUE][8];    // offsets per axis, momenta, charge
    __shared__ int sNleave;
    __shared__ int sChunk;   // DYN: next chunk of the current species
    // per-warp energy of every species, summed when the tile is done
    __shared__ float sEne[MAX_TILED_SPECIES][8];
    if (threadIdx.x == 0) {
        sNleave = 0;
        sChunk = 0;
    }
    __syncthreads();

    const int esy = 3 * ee[0], esz = 3 * ee[0] * ee[1];
    const unsigned lane = threadIdx.x & 31;
    float *sJw = DIM == 2 ? sJ + 3 * nj * warp : sJ;
    ColSlots<ORD> cs;
    if constexpr (DIM == 2) cs.init(jsy);

    SegRec *sQ = sQ0 + warp * QCAP;
    scr += warp * SCRF;
    int qn = 0;

    for (int s = 0; s < a.nspec; s++) {
        const SpeciesDev sd = a.spec[s];
        const long cap = sd.cap;
        const long slab = tile * cap;
        const int nst = min(sd.in.cnt[tile], (int)cap);
        const int nar = min(sd.in.arr[tile], (int)cap - nst);
        const int n = nst + nar;
        int *hist = sHist + (s & 1) * ncell;
        // per-thread partial energy in FP32 (the reference sums in single precision per
        // 464-particle chunk), summed per warp and per tile in FP32, across tiles in double
        float my_ene = 0.f;
        // ---- pass A: push every particle of the tile.  Particles that stay are written back
        //      to their own slot of the input slab (this CTA owns it) and counted per new cell,
        //      their sort key (new cell in the tile, rank among that cell's stayers) in place
        //      of the first cell index;
        //      particles that leave take an arrival slot (from the top) of their destination
        //      tile in the output buffer, and their input slot is marked empty (ix = 0).
        auto slot = [&](int i) { return slab + (i < nst ? i : cap - 1 - (i - nst)); };
        // the particle of the next iteration is loaded while this one is pushed
        int pf_c[3] = {1, 1, 1};
        float pf_x[3] = {0, 0, 0}, pf_u[3] = {0, 0, 0}, pf_q = 0.0f;
        float *const rin = sd.in.rec;
        auto prefetch = [&](int i, int lim) {
            if (i < lim) {
                load_rec<DIM>(rin, slot(i), pf_c, pf_x, pf_u, pf_q);
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
                    *rec_ix0<DIM>(rin, p) = 0;
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
                if constexpr (DIM == 2)
                    gather_tile2_paired<ORD>(sE, sB, esy, lf, lh, w, wh, E1, E2, E3, B1, B2, B3);
                else
                    gather_tile<DIM, ORD>(sE, sB, esy, esz, lf, lh, w, wh, E1, E2, E3, B1, B2, B3);
                if constexpr (PUSHER == OSG_PUSHER_EXACT) {
                    my_ene += exact_push<float>(sd.qm, a.dt_full, a.iter_tol, E1, E2, E3, B1,
                                                B2, B3, q, un[0], un[1], un[2]);
                } else if constexpr (PUSHER == OSG_PUSHER_VAY) {
                    my_ene += vay_push<float>(sd.tem, E1, E2, E3, B1, B2, B3, q, un[0], un[1],
                                              un[2]);
                } else if constexpr (PUSHER == OSG_PUSHER_HC) {
                    my_ene += (float)hc_push<float>(sd.tem, E1, E2, E3, B1, B2, B3, q, un[0],
                                                    un[1], un[2]);
                } else if constexpr (PUSHER == OSG_PUSHER_FULLROT) {
                    my_ene += (float)fullrot_push<float>(sd.tem, E1, E2, E3, B1, B2, B3, q,
                                                         un[0], un[1], un[2]);
                } else if constexpr (PUSHER == OSG_PUSHER_EULER) {
                    my_ene += (float)euler_push<float>(sd.tem, sd.rqm, a.dt_full, E1, E2, E3, B1,
                                                       B2, B3, q, un[0], un[1], un[2]);
                } else if constexpr (PUSHER == OSG_PUSHER_COND_VAY) {
                    my_ene += (float)cond_vay_push<float>(sd.tem, E1, E2, E3, B1, B2, B3, q,
                                                          un[0], un[1], un[2]);
                } else {
                    const float ene = boris(sd.tem, E1, E2, E3, B1, B2, B3, un[0], un[1], un[2]);
                    my_ene = fmaf(q, ene, my_ene);
                }
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
                int cn[3];
#pragma unroll
                for (int d = 0; d < DIM; d++) {
                    xo[d] = x1[d] - float(di[d]);
                    cn[d] = c[d] + di[d];
                    cw[d] = wrapc(cn[d], a.nx[d]);
                }
                // non-periodic axes (a launch-uniform test, so the periodic box pays one branch)
                bool gone = false;
                if (a.walls | a.open | a.window) {
                    int tb = 0;   // thermal-bath edges crossed (2 bits per axis)
#pragma unroll
                    for (int d = 0; d < DIM; d++) {
                        if (BATH && ((a.thermal >> d) & 1)) {
                            // thermal bath: re-emitted from the edge below
                            cw[d] = cn[d];
                            if (cn[d] < 1 || cn[d] > a.nx[d])
                                tb |= (cn[d] < 1 ? 1 : 2) << (2 * d);
                        } else if ((a.walls >> d) & 1) {
                            // conducting wall: specular reflection after the deposit of the
                            // unreflected path (p_bc_specular,
                            // source/spec/os-spec-boundary.f03:1293-1310)
                            cw[d] = cn[d] < 1 ? 1 : (cn[d] > a.nx[d] ? a.nx[d] : cn[d]);
                            if (cw[d] != cn[d]) {
                                xo[d] = -xo[d];
                                un[d] = -un[d];
                            }
                        } else if (d == 0 && a.window) {
                            // moving window along x1: the upper edge reflects specularly
                            // (p_bc_move_c behaves as p_bc_specular there, source/spec/
                            // os-spec-boundary.f03:1276, 1293-1310), the lower one absorbs
                            // (:315); a particle is stored one cell lower when the step ends
                            // with a window move and leaves when that puts it below cell 1
                            int cx = cn[0];
                            if (cx > a.nx[0]) {
                                cx = a.nx[0];
                                xo[0] = -xo[0];
                                un[0] = -un[0];
                            }
                            cw[0] = cx - a.shift_x;
                            gone = gone || cn[0] < 1 || cw[0] < 1;
                        } else if ((a.open >> d) & 1) {
                            // open axis (Lindman): a particle outside [1, nx] has left the
                            // box (absorbed); its current of this step is in the segments
                            cw[d] = cn[d];
                            gone = gone || cw[d] < 1 || cw[d] > a.nx[d];
                        }
                    }
                    if constexpr (BATH) {
                        if (tb)
                            tiled_reemit<DIM, ORD>(a, s, p, tb, t0, cn, cw, xo, un, q, sJw,
                                                   sJl, sJh, jsy, jsz);
                    }
                }
                if (gone) {
                    *rec_ix0<DIM>(rin, p) = 0;
                    has = false;
                } else {
                    // most particles stay in their tile: test that without dividing
                    bool inside = true;
#pragma unroll
                    for (int d = 0; d < DIM; d++)
                        inside = inside && cw[d] >= t0[d] && cw[d] < t0[d] + a.T[d];
                    if (inside) {
                        dest = tile;
                    } else {
#pragma unroll
                        for (int d = 0; d < DIM; d++) {
                            dt += mul * ((cw[d] - 1) / a.T[d]);
                            mul *= a.ntile[d];
                        }
                        dest = dt;
                    }
                }
            }
            const bool stay = has && dest == tile;
            int lcell = -1;
            if (stay) {
                lcell = cw[0] - t0[0];
                if (DIM > 1) lcell += a.T[0] * (cw[1] - t0[1]);
                if (DIM > 2) lcell += a.T[0] * a.T[1] * (cw[2] - t0[2]);
            }
            const unsigned peers = __match_any_sync(FULL_MASK, lcell);
            const int pl = __ffs(peers) - 1;
            int first = 0;
            if (stay && (int)lane == pl) first = atomicAdd(&hist[lcell], __popc(peers));
            first = __shfl_sync(FULL_MASK, first, pl);
            if (stay) {
                const int rank = first + __popc(peers & ((1u << lane) - 1u));
                const int kc[3] = {1 + lcell + (rank << SORT_CELL_BITS), cw[1], cw[2]};
                store_rec<DIM>(rin, p, kc, xo, un, q);
            }
            const bool leave = has && !stay;
            const unsigned ml = __ballot_sync(FULL_MASK, leave);
            if (ml) {
                const int leader = __ffs(ml) - 1;
                int q0 = 0;
                if ((int)lane == leader) q0 = atomicAdd(&sNleave, __popc(ml));
                q0 = __shfl_sync(FULL_MASK, q0, leader);
                if (leave) {
                    *rec_ix0<DIM>(rin, p) = 0;
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
            return nseg > 0 ? nseg : (has ? 0 : -1);
        };
        // a warp takes 32 consecutive particles of the cell-sorted tile (coalesced; mostly one
        // cell) at a time
        const int nck = (n + 31) >> 5;
        auto next_chunk = [&](int ck) {
            if constexpr (DYN) {
                int g = 0;
                if (lane == 0) g = atomicAdd(&sChunk, 1);
                return __shfl_sync(FULL_MASK, g, 0);
            } else {
                return ck < 0 ? warp : ck + nwarp;
            }
        };
        int ck = next_chunk(-1);
        if (ck < nck) prefetch(32 * ck + (int)lane, n);
        while (ck < nck) {
            const int i = 32 * ck + (int)lane;
            const int nk = next_chunk(ck);
            SegRec sg[MAXSEG];
            int c[3];
            float xo[3], un[3], q;
            take(c, xo, un, q);
            if (nk < nck) prefetch(32 * nk + (int)lane, n);
            const int ns = push_one(i < n, slot(i), c, xo, un, q, sg);
            if constexpr (BATH) __syncwarp();   // re-emission currents visible to the warp
            // ---- charge-conserving current of the segments into the shared tile: the first
            //      segment (in the particle's own cell, shared by neighbouring lanes of the
            //      cell-sorted tile) is summed per run of lanes with one cell; the others
            //      (face crossings, few and scattered) wait in the warp's queue for a
            //      full-warp deposit
#pragma unroll
            for (int t = 0; t < MAXSEG; t++) {
                const bool hs = t < ns;
                if constexpr (DIM == 2) {
                    if (t > 0) {
                        segq_push(sQ, qn, hs, sg[t]);
                        if (qn >= 32) segq_drain<ORD>(sJw, sQ, qn, 32, a.jn, scr, cs);
                        continue;
                    }
                    if (!__any_sync(FULL_MASK, hs)) break;
                    constexpr int NV = SegVals<2, ORD>::NV;
                    float v[NV];
                    if (hs) {
                        seg_values2_fast<ORD>(seg2_of<ORD>(sg[0]), q, a.jn[0], a.jn[1], v);
                    } else {
#pragma unroll
                        for (int k = 0; k < NV; k++) v[k] = 0.f;
                    }
                    cell_runs_deposit2<ORD>(sJw, jlo, scr, hs ? sg[0].base : -1, v, cs);
                } else {
                    if (t > 0) {
                        segq_push(sQ, qn, hs, sg[t]);
                        segq_drain3<ORD>(sJl, sJh, sQ, qn, SEGQ3_KEEP, a.jn, jsy, jsz,
                                         a.fx);
                        continue;
                    }
                    if (!__any_sync(FULL_MASK, hs)) break;
                    lanes_deposit3<ORD>(sJl, sJh, sg[0], hs, a.jn, jsy, jsz, a.fx);
                }
            }
            ck = nk;
        }
        // ---- energy: per-warp partial (the tile's sum is taken when the tile is done)
        {
            // FP32 (FP64 arithmetic runs at a small fraction of the FP32 rate on this GPU)
            float w = my_ene;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(FULL_MASK, w, o);
            if (lane == 0) sEne[s][warp] = w;
        }
        __syncthreads();   // the histogram and the leave queue are complete
        // ---- pass B (below) counting-sorts the particles that stayed into the output slab:
        //      offset of the cell + rank from the key, so that every step starts from particles
        //      in cell order (consecutive lanes share a cell).  No particle depends on another;
        //      every thread loads its first particle before the cell offsets are known, so the
        //      loads overlap the scan and the emigration (PB particles per thread and round:
        //      two or four spill registers and measured 3% and 8% slower)
        constexpr int PB = 1;
        long pp[PB];
        int key[PB], c1[PB], c2[PB];
        float xx[PB][DIM], uu[PB][3], qq[PB];
        auto pb_load = [&](int base) {
#pragma unroll
            for (int j = 0; j < PB; j++) {
                const int i = base + j * nthr + (int)threadIdx.x;
                pp[j] = slab + (i < nst ? i : cap - 1 - (i - nst));
                key[j] = 0;
                if (i < n) {
                    int cc[3];
                    float xr[3];
                    load_rec<DIM>(rin, pp[j], cc, xr, uu[j], qq[j]);
                    key[j] = cc[0];
                    c1[j] = DIM > 1 ? cc[1] : 0;
                    c2[j] = DIM > 2 ? cc[2] : 0;
#pragma unroll
                    for (int d = 0; d < DIM; d++) xx[j][d] = xr[d];
                }
            }
        };
        pb_load(0);
        // ---- warp 0: cell offsets of the particles that stayed; the other warps (meanwhile):
        //      the queued particles that left take their arrival slots; everyone: clear the
        //      next species' histogram
        {
            const int nq = min(sNleave, LEAVE_QUEUE);
            if (warp == 0) {
                const int nstay = warp_exclusive_scan(hist, ncell);
                if (threadIdx.x == 0) sd.out.cnt[tile] = nstay;
            }
            if (warp > 0 || nwarp == 1) {
                const int e0 = nwarp == 1 ? (int)threadIdx.x : (int)threadIdx.x - 32;
                const int es = nwarp == 1 ? nthr : nthr - 32;
                for (int e = e0; e < nq; e += es) {
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
            int *next = sHist + ((s + 1) & 1) * ncell;
            for (int k = threadIdx.x; k < ncell; k += nthr) next[k] = 0;
        }
        __syncthreads();
        // ---- pass B (the next particles are loaded before the current ones are stored)
        for (int base = 0; base < n; base += PB * nthr) {
            int ck[PB], cc1[PB], cc2[PB];
            float cx[PB][DIM], cu[PB][3], cq[PB];
#pragma unroll
            for (int j = 0; j < PB; j++) {
                ck[j] = key[j];
                cc1[j] = c1[j];
                cc2[j] = c2[j];
#pragma unroll
                for (int d = 0; d < DIM; d++) cx[j][d] = xx[j][d];
#pragma unroll
                for (int d = 0; d < 3; d++) cu[j][d] = uu[j][d];
                cq[j] = qq[j];
            }
            if (base + PB * nthr < n) pb_load(base + PB * nthr);
#pragma unroll
            for (int j = 0; j < PB; j++) {
                if (ck[j] > 0) {
                    const int kc = ck[j] - 1;
                    const int lc = kc & ((1 << SORT_CELL_BITS) - 1);
                    const long o = slab + hist[lc] + (kc >> SORT_CELL_BITS);
                    int ly = 0;
                    if (DIM > 1) ly = cc1[j] - t0[1];
                    if (DIM > 2) ly += a.T[1] * (cc2[j] - t0[2]);
                    const int oc[3] = {t0[0] + lc - a.T[0] * ly, cc1[j], cc2[j]};
                    store_rec<DIM, true>(sd.out.rec, o, oc, cx[j], cu[j], cq[j]);
                }
            }
        }
        if (threadIdx.x == 0) {
            sNleave = 0;
            sChunk = 0;
        }
        __syncthreads();
        if (a.discard) discard_dead_slab<DIM>(sd.in, slab, nst, nar, cap);
    }
    // ---- the face crossings still queued (the queue carries over from one species to the
    //      next: its entries hold their own charge)
    if constexpr (DIM == 2) segq_drain<ORD>(sJw, sQ, qn, 1, a.jn, scr, cs);
    else segq_drain3<ORD>(sJl, sJh, sQ, qn, 0, a.jn, jsy, jsz, a.fx);
    __syncthreads();
    // ---- the tile's energy of every species (the per-warp partials, written before the last
    //      block barrier)
    if ((int)threadIdx.x < a.nspec) {
        float tot = 0.f;
        for (int w = 0; w < nwarp; w++) tot += sEne[threadIdx.x][w];
        if (tot != 0.f) atomicAdd(a.ene + threadIdx.x, (double)tot);
    }
    // ---- store the tile's current (with halo) for the tile-ordered re-summation: in 2D the
    //      warp copies and their compensations summed into a float pair (hi, lo); in 3D the
    //      low and high words of the fixed-point tile
    {
        float *th = a.tile_hi + tile * (3L * nj);
        float *tl = a.tile_lo + tile * (3L * nj);
        for (int idx = threadIdx.x; idx < 3 * nj; idx += nthr) {
            if constexpr (DIM == 2) {
                // error-free FP32 cascade (two-sum of the running sum with every copy; the
                // errors and compensations summed apart), no FP64 arithmetic
                float hi = sJ[idx], lo = sJ[jlo + idx];
                for (int w = 1; w < nwarp; w++) {
                    const float v = sJ[3 * nj * w + idx], t = hi + v, bv = t - hi;
                    lo += ((hi - (t - bv)) + (v - bv)) + sJ[jlo + 3 * nj * w + idx];
                    hi = t;
                }
                const float t = hi + lo;
                th[idx] = t;
                tl[idx] = lo - (t - hi);
            } else {
                // the fixed-point words as they are (k_tile_fold sums them as integers), from
                // the padded rows
                const int pnt = idx / 3;
                const int sp = idx - 3 * pnt + 3 * (pnt % je[0]) + jsy * ((pnt / je[0]) % je[1]) +
                               jsz * (pnt / (je[0] * je[1]));
                th[idx] = __uint_as_float(sJl[sp]);
                tl[idx] = __uint_as_float(sJh[sp]);
            }
        }
    }
}

// Opt a push kernel in to `bytes` of dynamic shared memory (error if that does not fit beside
// its static shared memory).  The attribute belongs to the kernel, not to a state: it only
// grows, so that states of different tile shapes or CTA sizes in one process never lower it
// under one another.  (It is not raised to the device limit up front, which would let the
// driver size the L1/shared split for the largest launch possible rather than the one made.)
template <typename K> cudaError_t set_smem_room(K kernel, int bytes)
{
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, kernel);
    if (e != cudaSuccess) return e;
    int dev = 0, lim = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&lim, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev)) !=
        cudaSuccess)
        return e;
    if (bytes > lim - (int)fa.sharedSizeBytes) return cudaErrorInvalidValue;
    if (bytes <= fa.maxDynamicSharedSizeBytes) return cudaSuccess;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

template <int DIM, int ORD, int PUSHER, bool BATH>
__global__ void __launch_bounds__(256, push_min_blocks<DIM, ORD>()) k_push_tiled(TiledArgs a)
{
    push_tile<DIM, ORD, PUSHER, true, BATH>(a, blockIdx.x);
}

// launch of the single-box push: the thermal-bath variant when the state has a bath (Boris
// pusher only)
template <int D, int O, int P>
int launch_push_tiled(const TiledArgs &a, unsigned ntiles, int threads, size_t smem,
                      cudaStream_t st)
{
    if (a.thermal) {
        if constexpr (P == OSG_PUSHER_BORIS) {
            k_push_tiled<D, O, P, true><<<ntiles, threads, smem, st>>>(a);
            return OSG_OK;
        } else {
            set_error("tiled engine: the thermal bath runs with the Boris pusher");
            return OSG_ERR_ARG;
        }
    }
    k_push_tiled<D, O, P, false><<<ntiles, threads, smem, st>>>(a);
    return OSG_OK;
}

template <int D, int O, int P> cudaError_t attr_push_tiled(int bytes)
{
    cudaError_t e = set_smem_room(k_push_tiled<D, O, P, false>, bytes);
    if constexpr (P == OSG_PUSHER_BORIS)
        if (e == cudaSuccess) e = set_smem_room(k_push_tiled<D, O, P, true>, bytes);
    return e;
}

// Persistent push over many independent boxes in one launch: every CTA takes (box, tile)
// items from a work list (heaviest tiles first) through an atomic counter until the list is
// exhausted; the box's launch arguments are staged in shared memory per item.
template <int DIM, int ORD, int PUSHER>
__global__ void __launch_bounds__(256, push_min_blocks<DIM, ORD>())
k_push_tiled_batch(const TiledArgs *__restrict__ boxes, const int2 *__restrict__ work, int nwork,
                   int *counter)
{
    __shared__ TiledArgs sA;
    __shared__ int sItem;
    for (;;) {
        if (threadIdx.x == 0) sItem = atomicAdd(counter, 1);
        __syncthreads();
        const int it = sItem;
        if (it >= nwork) break;
        const int2 w = work[it];
        if (threadIdx.x == 0) sA = boxes[w.x];
        __syncthreads();
        push_tile<DIM, ORD, PUSHER, false, false>(sA, w.y);
        __syncthreads();
    }
}

// Deterministic current flush: every point of the global current (guard cells included) is
// the sum of the tile currents whose halo covers it, rounded once to float.  2D: FP64 sum, in
// increasing tile order, of the float pairs (hi + lo).  3D: exact 64-bit integer sum of the
// fixed-point tile values (from the words hi and lo, see tile_ops.cuh), converted with one
// rounding and scaled by fx_inv (a power of two) -- no FP64 arithmetic, whose rate is low on
// this GPU.  A tile with origin cell t0 = tc * T + 1 covers the global positions
// [tc * T - OFS + gcl, tc * T - OFS + gcl + je) along each axis (je = T + ORD + 2 points).
struct FoldBox {
    const float *th, *tl;   // tile currents (2D: value and compensation; 3D: fixed-point words)
    const int *empty;       // per tile: 1 = no particles this step, buffer not written
    float fx_inv;           // 3D: 1 / the fixed-point scale
    int fx_shift;           // 3D: bits of the low word
    float *j;               // global current
    int3 size, T, ntile, je, gcl;
    int ofs;
    long npts;              // 3 x grid points
};

// x / t for x >= 0, by a shift when t is a power of two (tile shapes always are in practice)
__device__ __forceinline__ int div_tile(int x, int t)
{
    return (t & (t - 1)) == 0 ? x >> (__ffs(t) - 1) : x / t;
}

// the folded value of component c at grid position (gx, gy, gz)
template <int DIM>
__device__ __forceinline__ float tile_fold_point(const float *__restrict__ th,
                                                 const float *__restrict__ tl,
                                                 const int *__restrict__ empty, int gx, int gy,
                                                 int gz, int c, int3 T, int3 ntile, int3 je,
                                                 int3 gcl, int ofs, float fx_inv, int fx_shift)
{
    const int gp[3] = {gx, gy, gz};
    const int Ta[3] = {T.x, T.y, T.z}, nt[3] = {ntile.x, ntile.y, ntile.z};
    const int jea[3] = {je.x, je.y, je.z}, gl[3] = {gcl.x, gcl.y, gcl.z};
    int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < 3; d++) {
        if (d < DIM) {
            // tiles tc with 0 <= gp - (tc * T - ofs + gl) < je
            const int r = gp[d] + ofs - gl[d];
            int a0 = r - jea[d] + 1;
            a0 = a0 <= 0 ? 0 : div_tile(a0 + Ta[d] - 1, Ta[d]);
            const int a1 = r < 0 ? -1 : div_tile(r, Ta[d]);
            lo[d] = a0;
            hi[d] = a1 < nt[d] - 1 ? a1 : nt[d] - 1;
        }
    }
    const int nj = jea[0] * (DIM > 1 ? jea[1] : 1) * (DIM > 2 ? jea[2] : 1);
    double v = 0.0;
    long long fx = 0;
    for (int tz = lo[2]; tz <= hi[2]; tz++)
        for (int ty = lo[1]; ty <= hi[1]; ty++)
            for (int tx = lo[0]; tx <= hi[0]; tx++) {
                const long tile = tx + (long)nt[0] * (ty + (long)nt[1] * tz);
                if (__ldg(empty + tile)) continue;
                const int lx = gx - (tx * Ta[0] - ofs + gl[0]);
                const int ly = DIM > 1 ? gy - (ty * Ta[1] - ofs + gl[1]) : 0;
                const int lz = DIM > 2 ? gz - (tz * Ta[2] - ofs + gl[2]) : 0;
                const long o = tile * (3L * nj) + 3 * (lx + jea[0] * (ly + jea[1] * lz)) + c;
                if constexpr (DIM == 3) {
                    // hi 2^B + (the low B bits of every add, summed: lo - hi 2^B mod 2^32)
                    const int hw = __float_as_int(tl[o]);
                    const unsigned lw = __float_as_uint(th[o]) - ((unsigned)hw << fx_shift);
                    fx += (long long)hw * (1LL << fx_shift) + (long long)lw;
                } else {
                    v += (double)th[o];
                    if (tl) v += (double)tl[o];
                }
            }
    if constexpr (DIM == 3) return __ll2float_rn(fx) * fx_inv;
    else return (float)v;
}

// single box: one grid row (3 components x size.x points) per (blockIdx.y, blockIdx.z) = (y, z),
// so no thread divides a 64-bit grid index
template <int DIM>
__global__ void k_tile_fold(const float *__restrict__ th, const float *__restrict__ tl,
                            const int *__restrict__ empty, float *__restrict__ j, int3 size,
                            int3 T, int3 ntile, int3 je, int3 gcl, int ofs, float fx_inv,
                            int fx_shift)
{
    const int gy = DIM > 1 ? (int)blockIdx.y : 0, gz = DIM > 2 ? (int)blockIdx.z : 0;
    const int row = 3 * size.x;
    float *jr = j + ((long)gz * size.y + gy) * row;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < row; i += gridDim.x * blockDim.x) {
        const int gx = i / 3;
        jr[i] = tile_fold_point<DIM>(th, tl, empty, gx, gy, gz, i - 3 * gx, T, ntile, je, gcl,
                                     ofs, fx_inv, fx_shift);
    }
}

// the same for every box of a batch: box = blockIdx.z, grid row (y, z) = blockIdx.y (rows
// past the box's last one exit at once)
template <int DIM>
__global__ void k_batch_fold(const FoldBox *__restrict__ boxes)
{
    const FoldBox &f = boxes[blockIdx.z];
    const int rows = f.size.y * (DIM > 2 ? f.size.z : 1);
    if ((int)blockIdx.y >= rows) return;
    const int gy = DIM > 1 ? (int)blockIdx.y % f.size.y : 0;
    const int gz = DIM > 2 ? (int)blockIdx.y / f.size.y : 0;
    const int row = 3 * f.size.x;
    float *jr = f.j + (long)blockIdx.y * row;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < row; i += gridDim.x * blockDim.x) {
        const int gx = i / 3;
        jr[i] = tile_fold_point<DIM>(f.th, f.tl, f.empty, gx, gy, gz, i - 3 * gx, f.T, f.ntile,
                                     f.je, f.gcl, f.ofs, f.fx_inv, f.fx_shift);
    }
}

// zero n ints at p for every range of a device table (one launch; defined in tiled.cu)
struct IntRange {
    int *p;
    long n;
};
void zero_ranges(const IntRange *d_ranges, int nrange, long max_n, cudaStream_t st);
// batched fold of the tile currents of every box (defined in tiled.cu)
void batch_fold(const FoldBox *d_boxes, int nbox, int dim, int max_row, int max_rows,
                cudaStream_t st);
// CTAs of the batched push resident per SM (defined in batch_push.cu)
int push_batch_occupancy(int dim, int order, int threads, size_t smem);

// Moving window: cold particles of one species in the new last x1 plane of cells (cells
// (nx1, j, k)), ppc[d] per cell on the OSIRIS lattice, charge sign(1/ppc, rqm) * den with den
// the piecewise-linear profile (prof_x, prof_f: n points, linear between them, 0 outside) at
// the particle's global x1 = (moved + i1 - 0.5 + offset) * dx1, where moved counts the window
// moves so far (injection of inject_std, source/spec/psource/os-psource-std.f03:759-1120; the
// piecewise-linear profile :23).  Cells where den <= 0 get no particles.  New particles take
// arrival slots (from the top) of their tile in the buffer the push just wrote.
struct InjectArgs {
    Slabs out;
    long cap;
    int T[3], ntile[3], nx[3], ppc[3], dim;
    double dx1, charge_unit;
    int nprof;
    double prof_x[8], prof_f[8];
    const int *moved;
    int *status;
};

__device__ __forceinline__ double profile_pl(const InjectArgs &a, double x)
{
    if (a.nprof <= 0 || x < a.prof_x[0] || x > a.prof_x[a.nprof - 1]) return 0.0;
    for (int k = 1; k < a.nprof; k++)
        if (x <= a.prof_x[k]) {
            const double w = (x - a.prof_x[k - 1]) / (a.prof_x[k] - a.prof_x[k - 1]);
            return a.prof_f[k - 1] + w * (a.prof_f[k] - a.prof_f[k - 1]);
        }
    return a.prof_f[a.nprof - 1];
}

template <int DIM>
__global__ void k_inject_x(InjectArgs a)
{
    const int py = DIM > 1 ? a.ppc[1] : 1, pz = DIM > 2 ? a.ppc[2] : 1;
    const int per = a.ppc[0] * py * pz;
    const int ny = DIM > 1 ? a.nx[1] : 1, nz = DIM > 2 ? a.nx[2] : 1;
    const long n = (long)ny * nz * per;
    const int moved = *a.moved;
    OSG_GRID_LOOP(g, n)
    {
        const int sub = (int)(g % per);
        const long cell = g / per;
        const int cj = 1 + (int)(cell % ny), ck = 1 + (int)(cell / ny);
        const int sa = sub / (py * pz), sb = (sub / pz) % py, sc = sub % pz;
        const int sidx[3] = {sa, sb, sc};
        float off[3];
#pragma unroll
        for (int d = 0; d < 3; d++) {
            const float half = 0.5f / (float)a.ppc[d];
            off[d] = (float)(2 * (sidx[d] + 1) - 1 - a.ppc[d]) * half;
        }
        const double xg = ((double)moved + a.nx[0] - 0.5 + (double)off[0]) * a.dx1;
        const float den = (float)profile_pl(a, xg);
        if (!(den > 0.0f)) continue;
        const int cw[3] = {a.nx[0], cj, ck};
        long tile = 0, mul = 1;
#pragma unroll
        for (int d = 0; d < DIM; d++) {
            tile += mul * ((cw[d] - 1) / a.T[d]);
            mul *= a.ntile[d];
        }
        const int k = atomicAdd(a.out.arr + tile, 1);
        const int room = (int)a.cap - min(a.out.cnt[tile], (int)a.cap);
        if (k >= room) {
            atomicOr(a.status, OSG_STATUS_OVERFLOW);
            continue;
        }
        const float u0[3] = {0.0f, 0.0f, 0.0f};
        store_rec<DIM>(a.out.rec, tile * a.cap + a.cap - 1 - k, cw, off, u0,
                       den * (float)a.charge_unit);
    }
}

// count of window moves (device counter read by the injection)
__global__ void k_count_move(int *moved);

// Launch of the push kernel of one (dim, order) for each pusher, and the opt-in to its dynamic
// shared memory (call outside stream capture).  tiled.cu defines the Boris pair, tiled_exact.cu
// the exact-pusher pair, tiled_vay.cu, tiled_hc.cu, tiled_fullrot.cu and tiled_euler.cu the
// other pushers' pairs (one unit each, so they compile in parallel).
int push_tiled_launch_boris(int dim, int order, const TiledArgs &a, unsigned ntiles,
                            int threads, size_t smem, cudaStream_t st);
cudaError_t push_tiled_attr_boris(int dim, int order, int bytes);
int push_tiled_launch_exact(int dim, int order, const TiledArgs &a, unsigned ntiles,
                            int threads, size_t smem, cudaStream_t st);
cudaError_t push_tiled_attr_exact(int dim, int order, int bytes);
int push_tiled_launch_vay(int dim, int order, const TiledArgs &a, unsigned ntiles, int threads,
                          size_t smem, cudaStream_t st);
cudaError_t push_tiled_attr_vay(int dim, int order, int bytes);
int push_tiled_launch_hc(int dim, int order, const TiledArgs &a, unsigned ntiles, int threads,
                         size_t smem, cudaStream_t st);
cudaError_t push_tiled_attr_hc(int dim, int order, int bytes);
int push_tiled_launch_fullrot(int dim, int order, const TiledArgs &a, unsigned ntiles,
                              int threads, size_t smem, cudaStream_t st);
cudaError_t push_tiled_attr_fullrot(int dim, int order, int bytes);
int push_tiled_launch_euler(int dim, int order, const TiledArgs &a, unsigned ntiles, int threads,
                            size_t smem, cudaStream_t st);
cudaError_t push_tiled_attr_euler(int dim, int order, int bytes);
int push_tiled_launch_cond_vay(int dim, int order, const TiledArgs &a, unsigned ntiles,
                               int threads, size_t smem, cudaStream_t st);
cudaError_t push_tiled_attr_cond_vay(int dim, int order, int bytes);
// persistent launch over a (box, tile) work list (k_push_tiled_batch, Boris pusher; defined
// in batch_push.cu)
int push_batch_launch(int dim, int order, const TiledArgs *boxes, const int2 *work, int nwork,
                      int *counter, unsigned grid, int threads, size_t smem, cudaStream_t st);
cudaError_t push_batch_attr(int dim, int order, int bytes);

#define OSG_DEFINE_PUSH_TILED(P, LAUNCH, ATTR)                                                \
    int LAUNCH(int dim, int order, const TiledArgs &a, unsigned ntiles, int threads,          \
               size_t smem, cudaStream_t st)                                                  \
    {                                                                                         \
        OSG_PUSH_TILED_CASES(P, OSG_PUSH_TILED_LAUNCH)                                        \
        set_error("tiled engine: unsupported dim %d order %d", dim, order);                  \
        return OSG_ERR_ARG;                                                                   \
    }                                                                                         \
    cudaError_t ATTR(int dim, int order, int bytes)                                           \
    {                                                                                         \
        OSG_PUSH_TILED_CASES(P, OSG_PUSH_TILED_ATTR)                                          \
        return cudaErrorInvalidValue;                                                         \
    }
#define OSG_DEFINE_PUSH_BATCH(P)                                                              \
    int push_batch_launch(int dim, int order, const TiledArgs *boxes, const int2 *work,       \
                          int nwork, int *counter, unsigned grid, int threads, size_t smem,   \
                          cudaStream_t st)                                                    \
    {                                                                                         \
        OSG_PUSH_TILED_CASES(P, OSG_PUSH_BATCH_LAUNCH)                                        \
        set_error("batched engine: unsupported dim %d order %d", dim, order);                \
        return OSG_ERR_ARG;                                                                   \
    }                                                                                         \
    cudaError_t push_batch_attr(int dim, int order, int bytes)                                \
    {                                                                                         \
        OSG_PUSH_TILED_CASES(P, OSG_PUSH_BATCH_ATTR)                                          \
        return cudaErrorInvalidValue;                                                         \
    }
#define OSG_PUSH_TILED_LAUNCH(D, O, P)                                                        \
    if (dim == D && order == O) return launch_push_tiled<D, O, P>(a, ntiles, threads, smem, st);
#define OSG_PUSH_TILED_ATTR(D, O, P)                                                          \
    if (dim == D && order == O) return attr_push_tiled<D, O, P>(bytes);
#define OSG_PUSH_BATCH_ATTR(D, O, P)                                                          \
    if (dim == D && order == O) return set_smem_room(k_push_tiled_batch<D, O, P>, bytes);
#define OSG_PUSH_BATCH_LAUNCH(D, O, P)                                                        \
    if (dim == D && order == O) {                                                             \
        k_push_tiled_batch<D, O, P><<<grid, threads, smem, st>>>(boxes, work, nwork, counter); \
        return OSG_OK;                                                                        \
    }
#define OSG_PUSH_TILED_CASES(P, X)                                                            \
    X(2, 1, P) X(2, 2, P) X(2, 3, P) X(2, 4, P) X(3, 1, P) X(3, 2, P) X(3, 3, P) X(3, 4, P)

} // namespace osg
