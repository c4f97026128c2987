// batch.cu -- many independent periodic boxes of uneven size and particle load advanced
// together (osg_batch_*).
//
// Every box is a tiled single-precision engine of its own (slabs, tile current buffers,
// fields), all with one tile shape.  One time step of the whole batch is a fixed sequence of
// launches, whatever the number of boxes, and is replayed from one CUDA graph per buffer
// parity:
//   E/B guard replace       batch_periodic (one launch per axis and field, all boxes)
//   push + deposit + sort   k_push_tiled_batch: a persistent grid (SMs x resident CTAs) takes
//                           (box, tile) items from a work list, heaviest boxes first, through
//                           an atomic counter, so large and small boxes share the GPU without
//                           a launch per box
//   current flush           batch_fold (FP64 tile-ordered re-summation, all boxes)
//   current guard fold      batch_periodic (add)
//   Yee                     batch_yee (B/2, E, B/2, all boxes)
// The phase order and the per-box arithmetic are those of the single-box tiled engine (the
// order of iter_sim, source/os-simulation.f03:498-666, per box).
//
// Autotuning: when the tile shape or the CTA size is left at 0, the first step times a proxy
// batch (one box of every distinct size and particle density) for every candidate tile shape
// and CTA size, and builds the batch with the fastest.  The tiled engine sorts every step (the
// sort is fused into the push), so there is no sort interval to tune.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <tuple>
#include <vector>

#include "common.cuh"
#include "fields.cuh"
#include "tiled.cuh"
#include "tiled_kernel.cuh"

namespace osg {

static const int BATCH_MAX_SPECIES = 16;

struct BatchSpecies {
    double rqm;
    long np;
    std::vector<int> ix;
    std::vector<float> x, u, q;
};

struct BatchBox {
    int nx[3] = {1, 1, 1};
    double dx[3] = {1, 1, 1};
    GridDesc g;
    std::vector<std::shared_ptr<const BatchSpecies>> sp;   // host copies (shared with proxies)
    TiledState *t = nullptr;
    float *e = nullptr, *b = nullptr, *j = nullptr;
    long np() const
    {
        long n = 0;
        for (const auto &s : sp) n += s->np;
        return n;
    }
};

} // namespace osg

using namespace osg;

struct osg_batch {
    osg_batch_config cfg;
    std::vector<BatchBox> box;
    cudaStream_t st = nullptr;
    bool built = false;
    int T[3] = {0, 0, 0};
    int threads = 0;
    int cur = 0;
    double *d_ene = nullptr;     // [box][BATCH_MAX_SPECIES]
    double *d_diag = nullptr;    // 6 doubles
    int *d_status = nullptr;
    int *d_counter = nullptr;
    TiledArgs *d_args[2] = {nullptr, nullptr};
    IntRange *d_zero[2] = {nullptr, nullptr};
    FieldBox *d_fb = nullptr;
    FoldBox *d_fold = nullptr;
    int2 *d_work = nullptr;
    int nwork = 0;
    unsigned grid = 0;
    size_t smem = 0;
    long max_side = 0, max_points = 0, max_cnt = 0;
    int max_row = 0, max_rows = 0;   // the fold's grid: 3 x size[0] values per row, rows
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    int launches = 0;
};

namespace osg {

static void free_built(osg_batch *b)
{
    for (auto &bx : b->box) {
        if (bx.t) tiled_destroy(bx.t);
        bx.t = nullptr;
        cudaFree(bx.e);
        cudaFree(bx.b);
        cudaFree(bx.j);
        bx.e = bx.b = bx.j = nullptr;
    }
    for (int p = 0; p < 2; p++) {
        cudaFree(b->d_args[p]);
        cudaFree(b->d_zero[p]);
        b->d_args[p] = nullptr;
        b->d_zero[p] = nullptr;
        if (b->graph[p]) cudaGraphExecDestroy(b->graph[p]);
        b->graph[p] = nullptr;
    }
    cudaFree(b->d_fb);
    cudaFree(b->d_fold);
    cudaFree(b->d_work);
    cudaFree(b->d_ene);
    cudaFree(b->d_diag);
    cudaFree(b->d_status);
    cudaFree(b->d_counter);
    b->d_fb = nullptr;
    b->d_fold = nullptr;
    b->d_work = nullptr;
    b->d_ene = b->d_diag = nullptr;
    b->d_status = b->d_counter = nullptr;
    b->built = false;
}

// device tables that hold pointers into the boxes (rebuilt after a box's slabs grow)
static int upload_tables(osg_batch *b)
{
    const int nb = (int)b->box.size();
    std::vector<TiledArgs> args[2];
    std::vector<IntRange> zero[2];
    std::vector<FieldBox> fb(nb);
    std::vector<FoldBox> fold(nb);
    for (int p = 0; p < 2; p++) {
        args[p].resize(nb);
        zero[p].resize(nb);
    }
    b->max_side = b->max_points = b->max_cnt = 0;
    b->max_row = b->max_rows = 0;
    for (int i = 0; i < nb; i++) {
        BatchBox &bx = b->box[i];
        for (int p = 0; p < 2; p++) {
            args[p][i] = tiled_args(bx.t, p, bx.e, bx.b, bx.j, b->d_ene + (size_t)i * BATCH_MAX_SPECIES,
                                    b->d_status);
            zero[p][i] = tiled_arrival_counters(bx.t, p);
        }
        fb[i] = make_field_box(bx.g, bx.e, bx.b, bx.j, bx.dx, b->cfg.dt);
        fold[i] = tiled_fold_box(bx.t, bx.j);
        b->max_points = std::max(b->max_points, bx.g.npoints());
        b->max_row = std::max(b->max_row, 3 * bx.g.size[0]);
        b->max_rows = std::max(b->max_rows, bx.g.size[1] * (bx.g.dim > 2 ? bx.g.size[2] : 1));
        b->max_cnt = std::max(b->max_cnt, zero[0][i].n);
        for (int d = 0; d < bx.g.dim; d++) {
            long other = 1;
            for (int a = 0; a < bx.g.dim; a++)
                if (a != d) other *= bx.g.size[a];
            b->max_side = std::max(b->max_side, other * (bx.g.gcl[d] + bx.g.gcu[d]));
        }
    }
    for (int p = 0; p < 2; p++) {
        OSG_CUDA(cudaMemcpy(b->d_args[p], args[p].data(), sizeof(TiledArgs) * nb, cudaMemcpyHostToDevice));
        OSG_CUDA(cudaMemcpy(b->d_zero[p], zero[p].data(), sizeof(IntRange) * nb, cudaMemcpyHostToDevice));
    }
    OSG_CUDA(cudaMemcpy(b->d_fb, fb.data(), sizeof(FieldBox) * nb, cudaMemcpyHostToDevice));
    OSG_CUDA(cudaMemcpy(b->d_fold, fold.data(), sizeof(FoldBox) * nb, cudaMemcpyHostToDevice));
    return OSG_OK;
}

static int enqueue_step(osg_batch *b, int parity, cudaStream_t st, int *launches)
{
    const int nb = (int)b->box.size(), dim = b->cfg.dim;
    int n = 0;
    batch_periodic(b->d_fb, nb, dim, 0, 0, b->max_side, st);
    batch_periodic(b->d_fb, nb, dim, 1, 0, b->max_side, st);
    n += 2 * dim;
    OSG_CUDA(cudaMemsetAsync(b->d_ene, 0, sizeof(double) * BATCH_MAX_SPECIES * nb, st));
    OSG_CUDA(cudaMemsetAsync(b->d_counter, 0, sizeof(int), st));
    zero_ranges(b->d_zero[parity], nb, b->max_cnt, st);
    n += 1;
    int rc = push_batch_launch(dim, b->cfg.order, b->d_args[parity], b->d_work, b->nwork,
                               b->d_counter, b->grid, b->threads, b->smem, st);
    if (rc) return rc;
    batch_fold(b->d_fold, nb, dim, b->max_row, b->max_rows, st);
    batch_periodic(b->d_fb, nb, dim, 2, 1, b->max_side, st);
    batch_yee(b->d_fb, nb, dim, b->max_points, st);
    n += 2 + dim + 3;
    OSG_CUDA(cudaGetLastError());
    if (launches) *launches = n;
    return OSG_OK;
}

static int capture(osg_batch *b)
{
    for (int p = 0; p < 2; p++) {
        if (b->graph[p]) cudaGraphExecDestroy(b->graph[p]);
        b->graph[p] = nullptr;
        cudaGraph_t gr;
        OSG_CUDA(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
        int rc = enqueue_step(b, p, b->st, &b->launches);
        cudaError_t ce = cudaStreamEndCapture(b->st, &gr);
        if (rc || ce != cudaSuccess) {
            if (ce == cudaSuccess) cudaGraphDestroy(gr);
            if (rc) return rc;
            OSG_CUDA(ce);
        }
        ce = cudaGraphInstantiate(&b->graph[p], gr, 0);
        cudaGraphDestroy(gr);
        OSG_CUDA(ce);
    }
    return OSG_OK;
}

// build every box with tile shape T and CTA size `threads` from the stored host particles
static int build(osg_batch *b, const int *T, int threads)
{
    free_built(b);
    const int nb = (int)b->box.size(), dim = b->cfg.dim;
    OSG_CHECK(nb > 0, OSG_ERR_STATE, "the batch has no boxes");
    for (int d = 0; d < 3; d++) b->T[d] = d < dim ? T[d] : 1;
    b->threads = threads;
    OSG_CUDA(cudaMalloc(&b->d_ene, sizeof(double) * BATCH_MAX_SPECIES * nb));
    OSG_CUDA(cudaMalloc(&b->d_diag, sizeof(double) * 6));
    OSG_CUDA(cudaMalloc(&b->d_status, sizeof(int)));
    OSG_CUDA(cudaMalloc(&b->d_counter, sizeof(int)));
    OSG_CUDA(cudaMemset(b->d_status, 0, sizeof(int)));
    for (int p = 0; p < 2; p++) {
        OSG_CUDA(cudaMalloc(&b->d_args[p], sizeof(TiledArgs) * nb));
        OSG_CUDA(cudaMalloc(&b->d_zero[p], sizeof(IntRange) * nb));
    }
    OSG_CUDA(cudaMalloc(&b->d_fb, sizeof(FieldBox) * nb));
    OSG_CUDA(cudaMalloc(&b->d_fold, sizeof(FoldBox) * nb));
    std::vector<std::pair<double, int>> weight;   // mean particles per tile, box
    for (int i = 0; i < nb; i++) {
        BatchBox &bx = b->box[i];
        osg_config c;
        memset(&c, 0, sizeof c);
        c.dim = dim;
        c.order = b->cfg.order;
        c.precision = 32;
        c.engine = OSG_ENGINE_TILED;
        for (int d = 0; d < 3; d++) {
            c.nx[d] = bx.nx[d];
            c.dx[d] = bx.dx[d];
            c.tile[d] = d < dim ? T[d] : 1;
        }
        c.dt = b->cfg.dt;
        c.capacity = b->cfg.capacity;
        c.pusher = OSG_PUSHER_BORIS;
        int rc = tiled_create(&bx.t, c, bx.g);
        if (rc) return rc;
        if ((rc = tiled_set_threads(bx.t, threads))) return rc;
        const size_t bytes = sizeof(float) * 3 * (size_t)bx.g.npoints();
        OSG_CUDA(cudaMalloc(&bx.e, bytes));
        OSG_CUDA(cudaMalloc(&bx.b, bytes));
        OSG_CUDA(cudaMalloc(&bx.j, bytes));
        OSG_CUDA(cudaMemset(bx.e, 0, bytes));
        OSG_CUDA(cudaMemset(bx.b, 0, bytes));
        OSG_CUDA(cudaMemset(bx.j, 0, bytes));
        for (const auto &s : bx.sp) {
            rc = tiled_add_species(bx.t, s->rqm, s->np, s->ix.data(), s->x.data(), s->u.data(),
                                   s->q.data(), b->st);
            if (rc) return rc;
        }
        weight.push_back({(double)bx.np() / (double)tiled_ntiles(bx.t), i});
    }
    b->smem = tiled_smem(b->box[0].t);
    const cudaError_t ae = push_batch_attr(dim, b->cfg.order, (int)b->smem);
    OSG_CHECK(ae == cudaSuccess, OSG_ERR_CUDA, "batched push: shared memory opt-in: %s",
              cudaGetErrorString(ae));
    // work list: every tile of every box, boxes with the heaviest tiles first
    std::stable_sort(weight.begin(), weight.end(),
                     [](const std::pair<double, int> &x, const std::pair<double, int> &y) {
                         return x.first > y.first;
                     });
    std::vector<int2> work;
    for (const auto &w : weight) {
        const long nt = tiled_ntiles(b->box[w.second].t);
        for (long k = 0; k < nt; k++) work.push_back(make_int2(w.second, (int)k));
    }
    OSG_CHECK(work.size() < (1u << 31), OSG_ERR_ARG, "too many tiles in the batch");
    b->nwork = (int)work.size();
    OSG_CUDA(cudaMalloc(&b->d_work, sizeof(int2) * work.size()));
    OSG_CUDA(cudaMemcpy(b->d_work, work.data(), sizeof(int2) * work.size(), cudaMemcpyHostToDevice));
    int dev = 0, nsm = 0;
    OSG_CUDA(cudaGetDevice(&dev));
    OSG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const int occ = push_batch_occupancy(dim, b->cfg.order, threads, b->smem);
    OSG_CHECK(occ > 0, OSG_ERR_ARG, "batched push does not fit on an SM (tile too large)");
    b->grid = (unsigned)std::min<long>((long)nsm * occ, b->nwork);
    b->cur = 0;
    int rc = upload_tables(b);
    if (rc) return rc;
    if ((rc = capture(b))) return rc;
    b->built = true;
    return OSG_OK;
}

static int run_steps(osg_batch *b, int nsteps)
{
    for (int s = 0; s < nsteps; s++) {
        OSG_CUDA(cudaGraphLaunch(b->graph[b->cur], b->st));
        b->cur ^= 1;
    }
    return OSG_OK;
}

static int check_after(osg_batch *b)
{
    int h = 0;
    OSG_CUDA(cudaMemcpyAsync(&h, b->d_status, sizeof(int), cudaMemcpyDeviceToHost, b->st));
    OSG_CUDA(cudaStreamSynchronize(b->st));
    OSG_CHECK(!(h & OSG_STATUS_RANGE), OSG_ERR_RANGE, "a particle left the valid cell range");
    OSG_CHECK(!(h & OSG_STATUS_OVERFLOW), OSG_ERR_OVERFLOW, "a tile ran out of particle slots");
    // grow the slabs of any box whose fullest tile passed 70% of its slots
    bool grown = false;
    for (auto &bx : b->box) {
        double f = 0.0;
        int rc = tiled_occupancy(bx.t, b->cur, &f, b->st);
        if (rc) return rc;
        if (f > 0.7) {
            if ((rc = tiled_regrow(bx.t, b->cur, b->st))) return rc;
            grown = true;
        }
    }
    if (grown) {
        int rc = upload_tables(b);
        if (rc) return rc;
        if ((rc = capture(b))) return rc;
    }
    return OSG_OK;
}

// Autotuner: time every candidate (tile shape x CTA size) on a proxy batch holding one box of
// every distinct (size, particles per cell) class, and keep the fastest.
static int autotune(osg_batch *b, int *bestT, int *best_threads)
{
    const int dim = b->cfg.dim;
    std::map<std::tuple<int, int, int, long>, int> classes;
    for (int i = 0; i < (int)b->box.size(); i++) {
        const BatchBox &bx = b->box[i];
        long cells = 1;
        for (int d = 0; d < dim; d++) cells *= bx.nx[d];
        const long ppc = (bx.np() + cells / 2) / cells;
        classes.emplace(std::make_tuple(bx.nx[0], bx.nx[1], bx.nx[2], ppc), i);
    }
    std::vector<std::array<int, 3>> tiles;
    if (dim == 2) tiles = {{8, 8, 1}, {16, 8, 1}, {16, 16, 1}};
    else tiles = {{4, 4, 4}, {8, 4, 4}, {8, 8, 4}};
    const int thr[2] = {256, 128};
    float best = 1e30f;
    bool found = false;
    for (const auto &T : tiles) {
        bool fits = true;
        for (const auto &bx : b->box)
            for (int d = 0; d < dim; d++)
                if (bx.nx[d] % T[d]) fits = false;
        if (!fits) continue;
        for (int th : thr) {
            osg_batch proxy;
            proxy.cfg = b->cfg;
            proxy.st = b->st;
            for (const auto &c : classes) proxy.box.push_back(b->box[c.second]);
            for (auto &bx : proxy.box) bx.t = nullptr, bx.e = bx.b = bx.j = nullptr;
            int rc = build(&proxy, T.data(), th);
            float ms = 0.0f;
            if (!rc) {
                rc = run_steps(&proxy, 2);
                cudaEvent_t e0, e1;
                cudaEventCreate(&e0);
                cudaEventCreate(&e1);
                cudaEventRecord(e0, proxy.st);
                if (!rc) rc = run_steps(&proxy, 3);
                cudaEventRecord(e1, proxy.st);
                if (cudaEventSynchronize(e1) != cudaSuccess) rc = OSG_ERR_CUDA;
                cudaEventElapsedTime(&ms, e0, e1);
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
            }
            proxy.st = nullptr;
            free_built(&proxy);
            if (rc == OSG_ERR_CUDA) return rc;
            if (rc) continue;   // candidate does not fit (shared memory, ...)
            if (ms < best) {
                best = ms;
                for (int d = 0; d < 3; d++) bestT[d] = T[d];
                *best_threads = th;
                found = true;
            }
        }
    }
    OSG_CHECK(found, OSG_ERR_ARG, "autotuner: no tile shape divides every box");
    return OSG_OK;
}

static int ensure_built(osg_batch *b)
{
    if (b->built) return OSG_OK;
    int T[3] = {b->cfg.tile[0], b->cfg.tile[1], b->cfg.tile[2]};
    int th = b->cfg.threads;
    bool tune = th == 0;
    for (int d = 0; d < b->cfg.dim; d++) tune = tune || T[d] <= 0;
    if (tune) {
        int bt[3] = {8, 8, 1}, bth = 256;
        int rc = autotune(b, bt, &bth);
        if (rc) return rc;
        for (int d = 0; d < 3; d++)
            if (T[d] <= 0) T[d] = bt[d];
        if (th == 0) th = bth;
    }
    return build(b, T, th);
}

} // namespace osg

extern "C" {

int osg_batch_create(const osg_batch_config *cfg, osg_batch **out)
{
    OSG_CHECK(cfg && out, OSG_ERR_ARG, "null argument");
    *out = nullptr;
    OSG_CHECK(cfg->dim == 2 || cfg->dim == 3, OSG_ERR_ARG, "dim must be 2 or 3");
    OSG_CHECK(cfg->order >= 1 && cfg->order <= 4, OSG_ERR_ARG, "order must be 1..4");
    OSG_CHECK(cfg->dt > 0, OSG_ERR_ARG, "dt must be positive");
    OSG_CHECK(cfg->threads == 0 || (cfg->threads >= 64 && cfg->threads <= 256 &&
                                    cfg->threads % 32 == 0),
              OSG_ERR_ARG, "threads must be 0 or a multiple of 32 in [64, 256]");
    osg_batch *b = new osg_batch();
    b->cfg = *cfg;
    if (cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess) {
        delete b;
        set_error("no CUDA device / stream creation failed");
        return OSG_ERR_CUDA;
    }
    *out = b;
    return OSG_OK;
}

int osg_batch_destroy(osg_batch *b)
{
    if (!b) return OSG_OK;
    if (b->st) cudaStreamSynchronize(b->st);
    free_built(b);
    if (b->st) cudaStreamDestroy(b->st);
    delete b;
    return OSG_OK;
}

int osg_batch_add_box(osg_batch *b, const int *nx, const double *dx)
{
    OSG_CHECK(b && nx && dx, OSG_ERR_ARG, "null argument");
    OSG_CHECK(!b->built, OSG_ERR_STATE, "boxes must be added before the first step");
    const int dim = b->cfg.dim;
    BatchBox bx;
    double cour = 0.0;
    for (int d = 0; d < dim; d++) {
        OSG_CHECK(nx[d] >= 2 * b->cfg.order + 1 && dx[d] > 0, OSG_ERR_ARG,
                  "nx[%d] too small or dx <= 0", d);
        bx.nx[d] = nx[d];
        bx.dx[d] = dx[d];
        cour += 1.0 / (dx[d] * dx[d]);
    }
    // Courant condition of the Yee solver (source/emf/solver/os-emf-solver-yee.f03:430-456)
    OSG_CHECK(b->cfg.dt <= std::sqrt(1.0 / cour), OSG_ERR_ARG,
              "dt violates the Yee Courant limit %g of this box", std::sqrt(1.0 / cour));
    int gl, gu;
    guard_cells(b->cfg.order, &gl, &gu);
    const int gcl[3] = {gl, gl, gl}, gcu[3] = {gu, gu, gu};
    bx.g = make_grid(dim, bx.nx, gcl, gcu);
    b->box.push_back(std::move(bx));
    return (int)b->box.size() - 1;
}

int osg_batch_add_species(osg_batch *b, int box, double rqm, long np, const int *ix,
                          const float *x, const float *u, const float *q)
{
    OSG_CHECK(b && box >= 0 && box < (int)b->box.size(), OSG_ERR_ARG, "bad box");
    OSG_CHECK(!b->built, OSG_ERR_STATE, "species must be added before the first step");
    OSG_CHECK(np >= 0 && (np == 0 || (ix && x && u && q)), OSG_ERR_ARG, "bad particle arrays");
    BatchBox &bx = b->box[box];
    OSG_CHECK((int)bx.sp.size() < BATCH_MAX_SPECIES, OSG_ERR_ARG, "too many species in a box");
    const int dim = b->cfg.dim;
    for (long p = 0; p < np; p++)
        for (int d = 0; d < dim; d++)
            OSG_CHECK(ix[dim * p + d] >= 1 && ix[dim * p + d] <= bx.nx[d], OSG_ERR_RANGE,
                      "particle %ld: cell index outside the box", p);
    auto s = std::make_shared<BatchSpecies>();
    s->rqm = rqm;
    s->np = np;
    s->ix.assign(ix, ix + (size_t)dim * np);
    s->x.assign(x, x + (size_t)dim * np);
    s->u.assign(u, u + (size_t)3 * np);
    s->q.assign(q, q + (size_t)np);
    bx.sp.push_back(std::move(s));
    return (int)bx.sp.size() - 1;
}

int osg_batch_tuning(osg_batch *b, int *tile, int *threads)
{
    OSG_CHECK(b, OSG_ERR_ARG, "null batch");
    int rc = ensure_built(b);
    if (rc) return rc;
    if (tile)
        for (int d = 0; d < 3; d++) tile[d] = b->T[d];
    if (threads) *threads = b->threads;
    return OSG_OK;
}

int osg_batch_step(osg_batch *b, int nsteps)
{
    OSG_CHECK(b && nsteps >= 0, OSG_ERR_ARG, "bad arguments");
    int rc = ensure_built(b);
    if (rc) return rc;
    if ((rc = run_steps(b, nsteps))) return rc;
    return check_after(b);
}

int osg_batch_time_steps(osg_batch *b, int nsteps, float *ms)
{
    OSG_CHECK(b && ms && nsteps > 0, OSG_ERR_ARG, "bad arguments");
    int rc = ensure_built(b);
    if (rc) return rc;
    cudaEvent_t e0, e1;
    OSG_CUDA(cudaEventCreate(&e0));
    OSG_CUDA(cudaEventCreate(&e1));
    cudaEventRecord(e0, b->st);
    rc = run_steps(b, nsteps);
    cudaEventRecord(e1, b->st);
    if (!rc && cudaEventSynchronize(e1) != cudaSuccess) rc = OSG_ERR_CUDA;
    if (!rc) cudaEventElapsedTime(ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc == OSG_ERR_CUDA) set_error("timed batch steps failed");
    if (rc) return rc;
    return check_after(b);
}

void *osg_batch_stream(osg_batch *b) { return b ? (void *)b->st : nullptr; }

int osg_batch_launches_per_step(osg_batch *b) { return b ? b->launches : 0; }

int osg_batch_num_boxes(osg_batch *b) { return b ? (int)b->box.size() : 0; }

int osg_batch_energy(osg_batch *b, int box, double *kinetic, double *field)
{
    OSG_CHECK(b && box >= 0 && box < (int)b->box.size(), OSG_ERR_ARG, "bad box");
    int rc = ensure_built(b);
    if (rc) return rc;
    BatchBox &bx = b->box[box];
    double dv = 1.0;
    for (int d = 0; d < b->cfg.dim; d++) dv *= bx.dx[d];
    if (kinetic) {
        double h[BATCH_MAX_SPECIES];
        OSG_CUDA(cudaMemcpyAsync(h, b->d_ene + (size_t)box * BATCH_MAX_SPECIES, sizeof h,
                                 cudaMemcpyDeviceToHost, b->st));
        OSG_CUDA(cudaStreamSynchronize(b->st));
        // get_energy normalisation, source/spec/os-spec-define.f03:1079-1084
        for (size_t k = 0; k < bx.sp.size(); k++) kinetic[k] = h[k] * bx.sp[k]->rqm * dv;
    }
    if (field) {
        OSG_CUDA(cudaMemsetAsync(b->d_diag, 0, 6 * sizeof(double), b->st));
        field_sumsq<float>(bx.g, bx.e, b->d_diag, b->st);
        field_sumsq<float>(bx.g, bx.b, b->d_diag + 3, b->st);
        OSG_CUDA(cudaGetLastError());
        double h[6];
        OSG_CUDA(cudaMemcpyAsync(h, b->d_diag, sizeof h, cudaMemcpyDeviceToHost, b->st));
        OSG_CUDA(cudaStreamSynchronize(b->st));
        for (int c = 0; c < 6; c++) field[c] = 0.5 * dv * h[c];
    }
    return OSG_OK;
}

int osg_batch_get_fields(osg_batch *b, int box, float *e, float *bf, float *j)
{
    OSG_CHECK(b && box >= 0 && box < (int)b->box.size(), OSG_ERR_ARG, "bad box");
    int rc = ensure_built(b);
    if (rc) return rc;
    BatchBox &bx = b->box[box];
    const size_t bytes = sizeof(float) * 3 * (size_t)bx.g.npoints();
    if (e) OSG_CUDA(cudaMemcpyAsync(e, bx.e, bytes, cudaMemcpyDeviceToHost, b->st));
    if (bf) OSG_CUDA(cudaMemcpyAsync(bf, bx.b, bytes, cudaMemcpyDeviceToHost, b->st));
    if (j) OSG_CUDA(cudaMemcpyAsync(j, bx.j, bytes, cudaMemcpyDeviceToHost, b->st));
    OSG_CUDA(cudaStreamSynchronize(b->st));
    return OSG_OK;
}

int osg_batch_num_particles(osg_batch *b, int box, int species, long *np)
{
    OSG_CHECK(b && np && box >= 0 && box < (int)b->box.size(), OSG_ERR_ARG, "bad box");
    int rc = ensure_built(b);
    if (rc) return rc;
    return tiled_count(b->box[box].t, b->cur, species, np, b->st);
}

int osg_batch_get_species(osg_batch *b, int box, int species, int *ix, float *x, float *u,
                          float *q)
{
    OSG_CHECK(b && box >= 0 && box < (int)b->box.size(), OSG_ERR_ARG, "bad box");
    int rc = ensure_built(b);
    if (rc) return rc;
    return tiled_get_species(b->box[box].t, b->cur, species, ix, x, u, q, b->st);
}

} // extern "C"
