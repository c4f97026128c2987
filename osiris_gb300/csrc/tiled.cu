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
// The per-particle arithmetic is the plain engine's (pic_math.cuh), i.e. the reference kernels'
// FNAME(vadvance_deposit_{2d,3d}_sN) (source/simd/os-spec-push-avx2.c:471-760, :1141-1480),
// except that the tiled kernels are compiled with the approximate single-precision division
// and square root (at most 2 ulp) and that the order in which current contributions are summed
// differs.  The migration and the per-step tile sort replace both the periodic particle
// boundary (source/spec/os-spec-boundary.f03:1280-1290) and the cell sort every n_sort steps
// (source/spec/os-species.f03:269-505).
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "fields.cuh"
#include "pic_math.cuh"
#include "push_plain.cuh"
#include "tiled.cuh"
#include "tiled_kernel.cuh"

namespace osg {

struct TiledState {
    int dim = 2, order = 2;
    int T[3] = {1, 1, 1}, ntile[3] = {1, 1, 1}, nx[3] = {1, 1, 1};
    long ntiles = 1;
    double capacity = 2.0;
    GridDesc g;
    double dt = 0, dx[3] = {1, 1, 1};
    std::vector<double> rqm;
    std::vector<long> cap;
    std::vector<double> qmax;   // per species: the largest |charge| a particle can carry
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
    // drop dead slab lines from L2 after the sort; OSG_L2_DISCARD=0 turns it off (profiler
    // kernel replay saves and restores device memory and needs the dropped lines defined)
    int l2_discard = 1;
    int walls = 0;   // bit d: conducting walls on axis d
    // thermal-bath particle boundary (bit d: walled or open axis d re-emits)
    int thermal = 0, thermal_type = 0;
    unsigned int seed = 0;
    float uth_bnd[3] = {0, 0, 0}, ufl_bnd[3] = {0, 0, 0};
    const unsigned long long *step = nullptr;   // the owner's step counter
    int open_fields = 0;   // bit d: Lindman or PML boundaries on axis d (particles absorbed)
    int pusher = OSG_PUSHER_BORIS;
    double iter_tol = 1.0e-3;
    long nj_tile = 0;    // current points (x3 components) of a tile with its halo
    float *tile_hi = nullptr, *tile_lo = nullptr;
    int *tile_empty = nullptr;   // per tile: no particles this step (written by the push)
    // moving window along x1 (open x1 boundary, injection into the new cells)
    bool window = false;
    int inj_species = -1;
    int inj_ppc[3] = {1, 1, 1};
    int nprof = 0;
    double prof_x[8] = {0}, prof_f[8] = {0};
    int *d_moved = nullptr;
    std::vector<long> min_cap;   // per species: at least this many slots per tile
};

OSG_DEFINE_PUSH_TILED(OSG_PUSHER_BORIS, push_tiled_launch_boris, push_tiled_attr_boris)

// --------------------------------------------------------------------------------- binning
// scatter particles (reference layout) to precomputed slab slots (host counting sort by tile
// and by cell inside the tile)
__global__ void k_bin(const int *__restrict__ ix, const float *__restrict__ x,
                      const float *__restrict__ u, const float *__restrict__ q,
                      const long *__restrict__ dst, long np, int dim, Slabs out)
{
    OSG_GRID_LOOP(p, np)
    {
        int c[3] = {0, 0, 0};
        float xo[3] = {0.f, 0.f, 0.f};
        for (int d = 0; d < dim; d++) {
            c[d] = ix[dim * p + d];
            xo[d] = x[dim * p + d];
        }
        const float un[3] = {u[3 * p], u[3 * p + 1], u[3 * p + 2]};
        if (dim == 2)
            store_rec<2>(out.rec, dst[p], c, xo, un, q[p]);
        else
            store_rec<3>(out.rec, dst[p], c, xo, un, q[p]);
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
        int c[3];
        float xo[3], un[3], qq;
        if (dim == 2)
            load_rec<2>(in.rec, src, c, xo, un, qq);
        else
            load_rec<3>(in.rec, src, c, xo, un, qq);
        for (int d = 0; d < dim; d++) {
            ix[dim * dst + d] = c[d];
            x[dim * dst + d] = xo[d];
        }
        u[3 * dst] = un[0];
        u[3 * dst + 1] = un[1];
        u[3 * dst + 2] = un[2];
        q[dst] = qq;
    }
}

// --------------------------------------------------------------------------------- host
// The single-precision SIMD push gets the time step rounded to p_k_part (dtcycle = real(dt,
// p_k_part), source/spec/os-spec-vpush.f03:365); the Fortran push the exact pusher runs in
// keeps the double dt (dt_dx = real(gdt/dx, p_k_part), source/spec/os-spec-push.f03:
// 1459-1460), as does the field solver.
static double push_dt(const TiledState *t)
{
    return t->pusher != OSG_PUSHER_BORIS ? t->dt : (double)(float)t->dt;
}

static cudaError_t push_attr(int pusher, int dim, int order, int bytes)
{
    switch (pusher) {
    case OSG_PUSHER_EXACT: return push_tiled_attr_exact(dim, order, bytes);
    case OSG_PUSHER_VAY: return push_tiled_attr_vay(dim, order, bytes);
    case OSG_PUSHER_HC: return push_tiled_attr_hc(dim, order, bytes);
    case OSG_PUSHER_FULLROT: return push_tiled_attr_fullrot(dim, order, bytes);
    case OSG_PUSHER_EULER: return push_tiled_attr_euler(dim, order, bytes);
    case OSG_PUSHER_COND_VAY: return push_tiled_attr_cond_vay(dim, order, bytes);
    default: return push_tiled_attr_boris(dim, order, bytes);
    }
}

// 3D fixed-point tile current.  A segment value is at most 3 |q| jn (weights along the motion
// <= |q| jn, across it <= 3); with a factor 2 of margin every value, times 2^S, is below
// V = 6 qmax jn 2^S in magnitude.  A tile point takes at most N adds per step: every particle
// of the tile's slabs (at most the sum of the capacities) adds one value per point for each of
// its at most 4 segments.  The low B bits of N values sum below 2^32: N 2^B <= 2^32.  The high
// word sums N values of magnitude <= V 2^-B + 1 and must stay below 2^31 - 1:
// V <= 2^B (2^31 / N - 2).  B is the largest with N 2^B <= 2^32, S the largest with V within
// both that bound and 2^31 (one value fits a signed 32-bit integer).  For N below 2^17 (slabs
// of up to 32768 slots in all) 2^S >= 2^28 / (6 qmax jn): each add rounds by at most 2^-29 of
// the largest value a segment can carry, far below the FP32 rounding of a float sum of
// currents of that order.  The quantum is absolute: currents many orders of magnitude below
// qmax jn (a cold plasma at rest) are resolved more coarsely than FP32 would.
static FxFormat fx_format(const TiledState *t)
{
    double jn = 0.0;
    for (int d = 0; d < t->dim; d++) jn = std::max(jn, t->dx[d] / push_dt(t) / 3.0);
    double qm = 0.0;
    for (double v : t->qmax) qm = std::max(qm, v);
    // segments per particle: 4 at most, plus 4 per re-emitting thermal-bath axis
    const double segs = 4.0 + 4.0 * __builtin_popcount((unsigned)t->thermal);
    double n = 0.0;
    for (long c : t->cap) n += segs * (double)c;
    n = std::max(n, 1.0);
    int B = (int)std::floor(32.0 - std::log2(n));
    while (B > 0 && n * std::ldexp(1.0, B) > 4294967296.0) B--;
    B = std::max(1, std::min(B, 30));
    const double vmax = std::min(2147483647.0, std::ldexp(1.0, B) * (2147483648.0 / n - 2.0));
    const double bound = 6.0 * qm * jn;
    int S = bound > 0.0 && vmax > 1.0 ? (int)std::floor(std::log2(vmax / bound)) : 40;
    FxFormat f;
    f.scale = std::ldexp(1.0f, std::max(-100, std::min(S, 100)));
    f.shift = B;
    return f;
}

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
    a.dt_full = t->dt;
    a.iter_tol = t->iter_tol;
    a.tile_hi = t->tile_hi;
    a.tile_lo = t->tile_lo;
    a.tile_empty = t->tile_empty;
    a.discard = t->l2_discard;
    a.walls = t->walls;
    a.thermal = t->thermal;
    a.thermal_type = t->thermal_type;
    a.seed = t->seed;
    a.step = t->step;
    for (int d = 0; d < 3; d++) {
        a.uth_bnd[d] = t->uth_bnd[d];
        a.ufl_bnd[d] = t->ufl_bnd[d];
    }
    a.fx = fx_format(t);
    return a;
}

// shared memory of the push kernel: E and B tiles and the current tile (one per warp with its
// compensation in 2D; the low and high words of the fixed-point tile in 3D)
static size_t smem_for(int dim, int order, const int *T, int threads)
{
    const int NP = order + 1;
    size_t ne = 1, nj = 1;
    for (int d = 0; d < dim; d++) {
        ne *= (size_t)(T[d] + NP);
        nj *= (size_t)(T[d] + NP + 1);
    }
    // 2D: one copy of the current tile per warp, each with its two-sum compensation, then per
    // warp a value scratch and a queue of face-crossing segments; last the cell histogram
    const size_t warps = (size_t)threads / 32;
    size_t jwords = 3 * nj * 2 * warps;
    if (dim == 3)
        jwords = 2 * ((size_t)(3 * (T[0] + NP + 1) + j3_pad_y(order)) * (T[1] + NP + 1) +
                      j3_pad_z(order)) *
                 (T[2] + NP + 1);
    const size_t nf = (6 * ne + jwords + 3) & ~(size_t)3;
    size_t cells = 1;
    for (int d = 0; d < dim; d++) cells *= (size_t)T[d];
    const size_t hist = 2 * cells * sizeof(int);
    if (dim != 2) return nf * sizeof(float) + warps * SEGQ3 * sizeof(SegRec) + hist;
    const int nv = 2 * order * NP + NP * NP;
    const size_t scratch = warps * (size_t)(nv + 1) * SCR_LD * sizeof(float);
    return nf * sizeof(float) + scratch + warps * SEGQ * sizeof(SegRec) + hist;
}

int tiled_create(TiledState **out, const osg_config &cfg, const GridDesc &g)
{
    TiledState *t = new TiledState();
    t->dim = cfg.dim;
    t->order = cfg.order;
    t->g = g;
    t->dt = cfg.dt;
    t->capacity = cfg.capacity > 0 ? cfg.capacity : 3.0;
    t->walls = cfg.walls;
    t->thermal = cfg.thermal;
    t->thermal_type = cfg.thermal_type;
    t->seed = cfg.seed;
    for (int d = 0; d < 3; d++) {
        t->uth_bnd[d] = (float)cfg.uth_bnd[d];
        t->ufl_bnd[d] = (float)cfg.ufl_bnd[d];
    }
    t->open_fields = cfg.open_fields | cfg.pml;   // particles absorbed along either
    t->ntiles = 1;
    for (int d = 0; d < 3; d++) {
        t->nx[d] = d < cfg.dim ? cfg.nx[d] : 1;
        t->dx[d] = cfg.dx[d];
        int T = 1;
        if (d < cfg.dim) {
            T = cfg.tile[d];
            if (T <= 0) {
                // 8 x 8 measured best on GB300 for 2D quadratic; 3D 8 x 8 x 4 (the deposit's
                // shared memory then allows two CTAs per SM)
                const int pref = (cfg.dim == 3 && d == 2) ? 4 : 8;
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
    if (const char *ev = getenv("OSG_L2_DISCARD")) t->l2_discard = atoi(ev) != 0;
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
    t->pusher = cfg.pusher;
    t->iter_tol = cfg.iter_tol > 0 ? cfg.iter_tol : 1.0e-3;
    // opt in to more than 48 KB of dynamic shared memory (outside any stream capture)
    {
        const cudaError_t ce = push_attr(t->pusher, t->dim, t->order, (int)t->smem_bytes);
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
    // per-tile current buffers of the deterministic flush (3 components x halo points)
    t->nj_tile = 3;
    for (int d = 0; d < t->dim; d++) t->nj_tile *= t->T[d] + t->order + 2;
    const size_t tb = sizeof(float) * (size_t)t->nj_tile * t->ntiles;
    if (cudaMalloc(&t->tile_hi, tb) != cudaSuccess || cudaMalloc(&t->tile_lo, tb) != cudaSuccess ||
        cudaMalloc(&t->tile_empty, sizeof(int) * t->ntiles) != cudaSuccess) {
        tiled_destroy(t);
        set_error("tile current allocation of %zu bytes failed", tb);
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
    cudaFree(t->tile_hi);
    cudaFree(t->tile_lo);
    cudaFree(t->tile_empty);
    cudaFree(t->d_moved);
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
            tab[k].tem = (float)pusher_tem(t->pusher, push_dt(t), (double)(float)t->rqm[k]);
            tab[k].rqm = (float)t->rqm[k];
            tab[k].qm = 1.0f / (float)t->rqm[k];
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
    if (k < (int)t->min_cap.size()) cap = std::max(cap, t->min_cap[k]);
    cap = (cap + 31) / 32 * 32;
    if (cap > MAX_TILE_SLOTS) {
        set_error("%ld particle slots per tile exceed the tile sort's limit of %ld: use smaller "
                  "tiles", cap, MAX_TILE_SLOTS);
        return OSG_ERR_ARG;
    }
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
        const size_t bytes = nslot * sizeof(float) * (dim == 2 ? PRec<2>::N : PRec<3>::N);
        char *mem = nullptr;
        if (cudaMalloc(&mem, bytes) != cudaSuccess) {
            set_error("particle slab allocation of %zu bytes failed", bytes);
            return OSG_ERR_NOMEM;
        }
        t->allocs.push_back(mem);
        // every tile's slab starts on a 128-byte line (the push drops dead lines from L2 by
        // address)
        if (((uintptr_t)mem & 127) != 0 || cap % 32 != 0) {
            set_error("particle slabs are not aligned to 128-byte lines");
            return OSG_ERR_CUDA;
        }
        s.rec = (float *)mem;
        s.cnt = t->d_cnt[p] + (size_t)k * t->ntiles;
        s.arr = t->d_arr[p] + (size_t)k * t->ntiles;
        OSG_CUDA(cudaMemsetAsync(s.arr, 0, sizeof(int) * t->ntiles, st));
        t->buf[p].push_back(s);
    }
    t->rqm.push_back(rqm);
    t->cap.push_back(cap);
    {
        // (a species re-binned by tiled_regrow keeps the bound it had)
        double qm = 0.0;
        for (long p = 0; p < np; p++) qm = std::max(qm, (double)std::fabs(q[p]));
        if (k < (int)t->qmax.size()) t->qmax[k] = std::max(qm, t->qmax[k]);
        else t->qmax.push_back(qm);
    }
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

TiledArgs tiled_args(TiledState *t, int parity, const float *e, const float *b, float *j,
                     double *d_ene, int *d_status)
{
    TiledArgs a = base_args(t);
    a.e = e;
    a.b = b;
    a.j = j;
    a.spec = t->d_tab[parity];
    a.nspec = (int)t->rqm.size();
    a.ene = d_ene;
    a.status = d_status;
    return a;
}

FoldBox tiled_fold_box(TiledState *t, float *j)
{
    const GridDesc &g = t->g;
    FoldBox f;
    f.th = t->tile_hi;
    f.tl = t->tile_lo;
    f.empty = t->tile_empty;
    f.j = j;
    f.size = make_int3(g.size[0], g.size[1], g.size[2]);
    f.T = make_int3(t->T[0], t->T[1], t->T[2]);
    f.ntile = make_int3(t->ntile[0], t->ntile[1], t->ntile[2]);
    f.je = make_int3(t->T[0] + t->order + 2, t->T[1] + t->order + 2, t->T[2] + t->order + 2);
    f.gcl = make_int3(g.gcl[0], g.gcl[1], g.gcl[2]);
    f.ofs = t->order == 1 ? 1 : (t->order == 4 ? 3 : 2);
    f.npts = 3 * g.npoints();
    const FxFormat fx = fx_format(t);
    f.fx_inv = 1.0f / fx.scale;
    f.fx_shift = fx.shift;
    return f;
}

IntRange tiled_arrival_counters(TiledState *t, int parity)
{
    IntRange r;
    r.p = t->d_arr[1 - parity];
    r.n = (long)MAX_TILED_SPECIES * t->ntiles;
    return r;
}

long tiled_ntiles(const TiledState *t) { return t->ntiles; }
size_t tiled_smem(const TiledState *t) { return t->smem_bytes; }
int tiled_threads(const TiledState *t) { return t->threads; }

__global__ void k_zero_ranges(const IntRange *__restrict__ r)
{
    const IntRange q = r[blockIdx.y];
    OSG_GRID_LOOP(i, q.n) q.p[i] = 0;
}

static unsigned grid_x(long n)
{
    long b = (n + 255) / 256;
    return (unsigned)(b < 1 ? 1 : (b > 1024 ? 1024 : b));
}

void zero_ranges(const IntRange *d_ranges, int nrange, long max_n, cudaStream_t st)
{
    k_zero_ranges<<<dim3(grid_x(max_n), (unsigned)nrange), 256, 0, st>>>(d_ranges);
}

void batch_fold(const FoldBox *d_boxes, int nbox, int dim, int max_row, int max_rows,
                cudaStream_t st)
{
    const dim3 grid((unsigned)((max_row + 255) / 256), (unsigned)max_rows, (unsigned)nbox);
    if (dim == 2) k_batch_fold<2><<<grid, 256, 0, st>>>(d_boxes);
    else k_batch_fold<3><<<grid, 256, 0, st>>>(d_boxes);
}

int tiled_set_step(TiledState *t, const unsigned long long *step)
{
    t->step = step;
    return OSG_OK;
}

int tiled_set_threads(TiledState *t, int threads)
{
    OSG_CHECK(threads >= 64 && threads <= 256 && threads % 32 == 0, OSG_ERR_ARG,
              "push CTA size must be a multiple of 32 in [64, 256]");
    t->threads = threads;
    t->smem_bytes = smem_for(t->dim, t->order, t->T, t->threads);
    const cudaError_t ce = push_attr(t->pusher, t->dim, t->order, (int)t->smem_bytes);
    OSG_CHECK(ce == cudaSuccess, OSG_ERR_CUDA, "cudaFuncSetAttribute: %s", cudaGetErrorString(ce));
    return OSG_OK;
}

__global__ void k_count_move(int *moved)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) *moved += 1;
}

bool tiled_window_params(const TiledState *t, int *species, int *ppc, int *nprof,
                         double *prof_x, double *prof_f)
{
    if (!t->window) return false;
    *species = t->inj_species;
    for (int d = 0; d < 3; d++) ppc[d] = t->inj_ppc[d];
    *nprof = t->nprof;
    for (int k = 0; k < 8; k++) {
        prof_x[k] = t->prof_x[k];
        prof_f[k] = t->prof_f[k];
    }
    return true;
}

int tiled_set_moves(TiledState *t, long moves, cudaStream_t st)
{
    OSG_CHECK(t->d_moved && moves >= 0 && moves <= INT_MAX, OSG_ERR_STATE, "no window");
    const int m = (int)moves;
    OSG_CUDA(cudaMemcpyAsync(t->d_moved, &m, sizeof(int), cudaMemcpyHostToDevice, st));
    OSG_CUDA(cudaStreamSynchronize(st));
    return OSG_OK;
}

int tiled_set_window(TiledState *t, int species, const int *ppc, int nprof,
                     const double *prof_x, const double *prof_f)
{
    OSG_CHECK(species >= 0 && species < (int)t->rqm.size(), OSG_ERR_ARG,
              "window injection: bad species");
    OSG_CHECK(nprof >= 1 && nprof <= 8 && prof_x && prof_f && ppc, OSG_ERR_ARG,
              "window injection: 1..8 profile points");
    for (int k = 1; k < nprof; k++)
        OSG_CHECK(prof_x[k] > prof_x[k - 1], OSG_ERR_ARG, "profile points must increase");
    for (int d = 0; d < t->dim; d++)
        OSG_CHECK(ppc[d] >= 1 && ppc[d] <= 64, OSG_ERR_ARG, "bad particles per cell");
    t->window = true;
    t->inj_species = species;
    for (int d = 0; d < 3; d++) t->inj_ppc[d] = d < t->dim ? ppc[d] : 1;
    t->nprof = nprof;
    for (int k = 0; k < nprof; k++) {
        t->prof_x[k] = prof_x[k];
        t->prof_f[k] = prof_f[k];
    }
    if (!t->d_moved) {
        OSG_CUDA(cudaMalloc(&t->d_moved, sizeof(int)));
        OSG_CUDA(cudaMemset(t->d_moved, 0, sizeof(int)));
    }
    // the injected plasma fills whole tiles: make room for 1.5 x a full tile
    long per_tile = 1, per = 1;
    for (int d = 0; d < t->dim; d++) {
        per_tile *= t->T[d];
        per *= t->inj_ppc[d];
    }
    const long need = (long)std::ceil(1.5 * (double)(per_tile * per)) + 64;
    // injected particles carry den / per, den at most the profile's largest value
    double fmax = 0.0;
    for (int k = 0; k < nprof; k++) fmax = std::max(fmax, std::fabs(prof_f[k]));
    t->qmax[species] = std::max(t->qmax[species], fmax / (double)per);
    if ((int)t->min_cap.size() < (int)t->rqm.size()) t->min_cap.resize(t->rqm.size(), 0);
    t->min_cap[species] = std::max(t->min_cap[species], need);
    if (t->cap[species] < need) return tiled_regrow(t, 0, 0);
    return OSG_OK;
}

// after a step that ended with a window move: count the move and inject the new x1 plane
// into the buffer the push wrote (1 - parity)
int tiled_window_inject(TiledState *t, int parity, int *d_status, cudaStream_t st,
                        int *launches)
{
    k_count_move<<<1, 32, 0, st>>>(t->d_moved);
    const int k = t->inj_species;
    InjectArgs a;
    memset(&a, 0, sizeof a);
    a.out = t->buf[1 - parity][k];
    a.cap = t->cap[k];
    a.dim = t->dim;
    int per = 1;
    for (int d = 0; d < 3; d++) {
        a.T[d] = t->T[d];
        a.ntile[d] = t->ntile[d];
        a.nx[d] = t->nx[d];
        a.ppc[d] = t->inj_ppc[d];
        if (d < t->dim) per *= t->inj_ppc[d];
    }
    a.dx1 = t->dx[0];
    a.charge_unit = (t->rqm[k] < 0 ? -1.0 : 1.0) * (double)(1.0f / (float)per);
    a.nprof = t->nprof;
    for (int i = 0; i < t->nprof; i++) {
        a.prof_x[i] = t->prof_x[i];
        a.prof_f[i] = t->prof_f[i];
    }
    a.moved = t->d_moved;
    a.status = d_status;
    const long n = (long)(t->dim > 1 ? t->nx[1] : 1) * (t->dim > 2 ? t->nx[2] : 1) * per;
    unsigned nb = blocks_for(n, 256);
    if (nb > 4096) nb = 4096;
    if (t->dim == 2) k_inject_x<2><<<nb, 256, 0, st>>>(a);
    else k_inject_x<3><<<nb, 256, 0, st>>>(a);
    *launches += 2;
    return OSG_OK;
}

int tiled_push(TiledState *t, int parity, const float *e, const float *b, float *j,
               double *d_ene, int *d_status, cudaStream_t st, int *launches, int shift)
{
    const int ns = (int)t->rqm.size();
    if (ns == 0) return OSG_OK;
    // the push writes every tile's sorted count and adds arrivals to zeroed counters
    OSG_CUDA(cudaMemsetAsync(t->d_arr[1 - parity], 0, sizeof(int) * MAX_TILED_SPECIES * t->ntiles, st));
    TiledArgs a = tiled_args(t, parity, e, b, j, d_ene, d_status);
    a.open = t->open_fields;
    a.window = t->window ? 1 : 0;
    a.shift_x = t->window && shift ? 1 : 0;
    const size_t sm = t->smem_bytes;
    const unsigned nt = (unsigned)t->ntiles;
    int rc;
    switch (t->pusher) {
    case OSG_PUSHER_EXACT: rc = push_tiled_launch_exact(t->dim, t->order, a, nt, t->threads, sm, st); break;
    case OSG_PUSHER_VAY: rc = push_tiled_launch_vay(t->dim, t->order, a, nt, t->threads, sm, st); break;
    case OSG_PUSHER_HC: rc = push_tiled_launch_hc(t->dim, t->order, a, nt, t->threads, sm, st); break;
    case OSG_PUSHER_FULLROT: rc = push_tiled_launch_fullrot(t->dim, t->order, a, nt, t->threads, sm, st); break;
    case OSG_PUSHER_EULER: rc = push_tiled_launch_euler(t->dim, t->order, a, nt, t->threads, sm, st); break;
    case OSG_PUSHER_COND_VAY:
        rc = push_tiled_launch_cond_vay(t->dim, t->order, a, nt, t->threads, sm, st);
        break;
    default: rc = push_tiled_launch_boris(t->dim, t->order, a, nt, t->threads, sm, st); break;
    }
    if (rc) return rc;
    // deterministic re-summation of the tile currents into the global current
    const FoldBox f = tiled_fold_box(t, j);
    const dim3 grid((unsigned)((3 * f.size.x + 255) / 256), (unsigned)f.size.y,
                    t->dim == 3 ? (unsigned)f.size.z : 1u);
    if (t->dim == 2)
        k_tile_fold<2><<<grid, 256, 0, st>>>(f.th, f.tl, f.empty, j, f.size, f.T, f.ntile, f.je,
                                             f.gcl, f.ofs, f.fx_inv, f.fx_shift);
    else
        k_tile_fold<3><<<grid, 256, 0, st>>>(f.th, f.tl, f.empty, j, f.size, f.T, f.ntile, f.je,
                                             f.gcl, f.ofs, f.fx_inv, f.fx_shift);
    *launches += 2;
    return OSG_OK;
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
    // the new slabs hold 1.5x the old ones at least: re-binning from the current counts alone
    // (1.25x the fullest tile) would leave a tile that triggered it 80% full
    if ((int)t->min_cap.size() < ns) t->min_cap.resize(ns, 0);
    for (int k = 0; k < ns && k < (int)t->cap.size(); k++)
        t->min_cap[k] = std::max(t->min_cap[k], (long)std::ceil(1.5 * (double)t->cap[k]));
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
