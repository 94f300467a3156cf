// serving.cuh -- zoom requests, batches and the serving loop (continuous
// batching).  Included once, by runtime.cu, after the session definition.
//
// A batch is a list of zoom requests (a cubic box and a resolution each)
// over the session's resident lattice.  Its work items pair a tile of a
// request grid (at most zoom_tile^3 cells) with a meta-cell whose AABB meets
// the tile.  Submitting builds the items on the host and queues the batch;
// it is ADMITTED when a device block of the session's arena and a stream are
// free, and then runs concurrently with the batches already on the GPU:
//
//   * memory: one arena per session (first-fit blocks inside a few large
//     cudaMalloc chunks, grown up to hbm_fraction of the HBM free at the
//     first submit and never returned until the session ends), so admitting
//     and finishing a batch make no cudaMalloc or cudaFree -- cudaFree
//     synchronises the whole device, which would make every finished batch
//     wait for every running one.  Results come back into pinned host blocks
//     of a second arena.
//   * streams: a fixed pool at three priorities; a batch's expected pair count
//     picks its priority (cheap batches higher), so the CTAs of a small
//     request take SMs ahead of the remaining CTAs of a large one.
//   * launch shape: one item per CTA (the persistent loop with
//     per_cta_items = 1), so a batch's CTAs leave the SMs as they finish and
//     concurrent batches share the GPU instead of queueing behind a grid that
//     holds every SM until its queue is empty.
//   * completion: a host function enqueued after the result copy stamps the
//     finish time and wakes the dispatcher thread, which frees the batch's
//     device block and stream and admits the batches waiting for them.
//
// Results are exact 64-bit fixed-point sums, so a request's masses are the
// same alone and in any mix.
#pragma once

#include <condition_variable>

namespace {

inline size_t round_up(size_t n, size_t a) { return (n + a - 1) / a * a; }

// Batches whose results take at most this many bytes get them back into
// pinned host memory with the launch; larger ones keep them on the device.
constexpr size_t kEagerBytes = size_t(1) << 30;

// expected-pair boundaries of the three priority classes of batches
constexpr double kClassPairs[2] = {1.6e7, 3.0e7};

// First-fit allocator over a few large chunks of device or pinned host memory.
struct Arena {
    struct Chunk {
        unsigned char *base = nullptr;
        size_t size = 0;
        std::map<size_t, size_t> free;  // offset -> size of each free range
    };
    struct Block {
        int chunk = -1;
        size_t off = 0, size = 0;
        unsigned char *ptr = nullptr;
    };
    std::vector<Chunk> chunks;
    size_t allocated = 0;   // bytes held in chunks
    size_t budget = 0;      // most bytes the chunks may hold
    size_t min_chunk = 0;   // a new chunk holds at least this much (within the budget)
    size_t live = 0;        // bytes handed out
    bool device = true;

    ~Arena()
    {
        for (Chunk &c : chunks) {
            if (device)
                cudaFree(c.base);
            else
                cudaFreeHost(c.base);
        }
    }

    static bool take(Chunk &c, int ci, size_t n, Block &b)
    {
        for (auto it = c.free.begin(); it != c.free.end(); ++it) {
            if (it->second < n) continue;
            b.chunk = ci;
            b.off = it->first;
            b.size = n;
            b.ptr = c.base + it->first;
            const size_t rest = it->second - n, roff = it->first + n;
            c.free.erase(it);
            if (rest) c.free[roff] = rest;
            return true;
        }
        return false;
    }

    // 0: allocated; 1: no room now (a later free may make room); else an
    // adeco_status_code (the message is set).
    int alloc(size_t n, Block &b)
    {
        n = round_up(std::max<size_t>(n, 1), 256);
        for (size_t i = 0; i < chunks.size(); ++i)
            if (take(chunks[i], (int)i, n, b)) {
                live += n;
                return 0;
            }
        if (allocated + n > budget) return 1;
        const size_t sz = std::max(n, std::min(min_chunk, budget - allocated));
        void *p = nullptr;
        const cudaError_t e = device ? cudaMalloc(&p, sz) : cudaHostAlloc(&p, sz, cudaHostAllocDefault);
        if (e != cudaSuccess) {
            cudaGetLastError();
            if (e == cudaErrorMemoryAllocation && live > 0) return 1;  // wait for blocks in use
            return fail(e == cudaErrorMemoryAllocation ? ADECO_ERR_MEMORY : ADECO_ERR_CUDA,
                        "serving arena: %s of %zu bytes failed: %s", device ? "cudaMalloc" : "cudaHostAlloc", sz,
                        cudaGetErrorString(e));
        }
        Chunk c;
        c.base = static_cast<unsigned char *>(p);
        c.size = sz;
        c.free[0] = sz;
        chunks.push_back(c);
        allocated += sz;
        take(chunks.back(), (int)chunks.size() - 1, n, b);
        live += n;
        return 0;
    }

    void release(Block &b)
    {
        if (b.chunk < 0) return;
        Chunk &c = chunks[b.chunk];
        size_t off = b.off, size = b.size;
        auto next = c.free.lower_bound(off);
        if (next != c.free.end() && off + size == next->first) {  // merge with the range after
            size += next->second;
            next = c.free.erase(next);
        }
        if (next != c.free.begin()) {  // merge with the range before
            auto prev = std::prev(next);
            if (prev->first + prev->second == off) {
                prev->second += size;
                live -= b.size;
                b = Block();
                return;
            }
        }
        c.free[off] = size;
        live -= b.size;
        b = Block();
    }
};

// Per request of a batch: first cell of its grid in the batch's output, cells, fixed-point scale.
struct ReqSlot {
    long long offset;
    long long cells;
    int shift;
    int pad[3];
};

// Fixed-point sums -> FP64 masses in place, each request with its own scale.
__global__ void requests_to_f64_kernel(unsigned long long *acc, const ReqSlot *req, int n_req, long long total)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        int lo = 0, hi = n_req - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (req[mid].offset <= i) lo = mid; else hi = mid - 1;
        }
        const double v = ldexp((double)acc[i], -req[lo].shift);
        reinterpret_cast<double *>(acc)[i] = v;
    }
}

}  // namespace

// Server is the type adeco_session points to (declared there at global scope).
struct Server;

struct ServeJob {
    uint64_t id = 0;
    Server *srv = nullptr;
    std::vector<adeco_request> reqs;
    std::vector<GridDesc> grids;   // one per tile of each request
    std::vector<Item> items;
    std::vector<ReqSlot> rtab;
    size_t cells = 0;
    double est_pairs = 0.0;        // expected candidate pairs (picks the priority)
    int level = 0;                 // stream priority class (0 highest)
    // block layout, identical on the device and in pinned memory up to off_route:
    // [results, cells x 8 B][status 16 B][request table][grid descriptors][items][route list]
    size_t off_stat = 0, off_req = 0, off_grids = 0, off_items = 0, off_route = 0, dev_bytes = 0;
    unsigned long long rcap = 0;
    // Results of at most kEagerBytes come back into the pinned block with the
    // launch (serving); larger batches keep them on the device until
    // adeco_session_result copies them, so the pinned block then holds only
    // the status words and inputs and starts at offset hoff = off_stat.
    bool eager = true;
    size_t hoff = 0;
    Arena::Block dblk, hblk;
    unsigned char *host(size_t off) const { return hblk.ptr + (off - hoff); }
    int stream = -1;               // index into the server's stream pool
    cudaEvent_t t0 = nullptr, t1 = nullptr;  // device time of its deposit launches
    std::chrono::steady_clock::time_point t_submit, t_done;
    int state = 0;                 // 0 queued, 1 on the GPU, 2 finished and finalised, 3 failed to launch
    std::atomic<int> done{0};      // set by the completion host function
    int err_bits = -1;             // device error flag, read from the status words once finished
    unsigned long long routed = 0;
    int fail_rc = 0;
    std::string fail_msg;
};

struct Server {
    adeco_session *s = nullptr;
    static constexpr int kLevels = 3, kPerLevel = 4;
    // streams a class may use at once: cheap batches share the GPU freely;
    // the most expensive class runs one batch at a time (first in, first
    // out), each at full speed, instead of several slowing each other down
    static constexpr int kUsable[kLevels] = {4, 2, 1};
    cudaStream_t streams[kLevels * kPerLevel] = {};
    bool stream_busy[kLevels * kPerLevel] = {};
    std::mutex mu;                 // jobs, queue, arenas, streams
    std::mutex cv_mu;              // only for the wake-ups (never held across CUDA calls)
    std::condition_variable cv;
    bool wake = false, stop = false;
    Arena dev, pin;
    std::deque<ServeJob *> pending;
    std::map<uint64_t, std::unique_ptr<ServeJob>> jobs;
    std::vector<ServeJob *> running_jobs;
    std::vector<cudaEvent_t> event_pool;
    uint64_t next_id = 1;
    double spacing = 1.0;          // mean lattice spacing (world units)
    std::thread dispatcher;
    adeco_serving_stats stats = {};

    void signal()
    {
        {
            std::lock_guard<std::mutex> lk(cv_mu);
            wake = true;
        }
        cv.notify_all();
    }
};

// Host function after a job's result copy: stamps the finish time and wakes
// the dispatcher.  It takes no lock that is ever held across a CUDA call.
static void CUDART_CB job_finished(void *arg)
{
    ServeJob *j = static_cast<ServeJob *>(arg);
    Server *S = j->srv;  // read first: once `done` is set the job may be released
    j->t_done = std::chrono::steady_clock::now();
    j->done.store(1, std::memory_order_release);
    S->signal();
}

// Frees a finished job's device block, stream and the waiting slot (mu held).
static void finalize_locked(Server &S, ServeJob &j)
{
    if (j.state != 1 || !j.done.load(std::memory_order_acquire)) return;
    const unsigned char *st = j.host(j.off_stat);
    int err = 0;
    unsigned long long routed = 0;
    std::memcpy(&err, st + 4, sizeof err);
    std::memcpy(&routed, st + 8, sizeof routed);
    j.err_bits = err;
    j.routed = routed;
    if (j.eager) S.dev.release(j.dblk);  // a lazy job's results stay until release
    S.stream_busy[j.stream] = false;
    j.state = 2;
    S.running_jobs.erase(std::find(S.running_jobs.begin(), S.running_jobs.end(), &j));
    S.stats.running = (uint32_t)S.running_jobs.size();
    ++S.stats.completed;
}

static cudaEvent_t take_event(Server &S)
{
    if (!S.event_pool.empty()) {
        cudaEvent_t e = S.event_pool.back();
        S.event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return e;
}

// Admits queued jobs that fit now (mu held): device and pinned blocks, a
// stream of the job's priority class, timing events.  FIFO, but a job that
// does not fit does not hold back the cheaper ones behind it.
static std::vector<ServeJob *> admit_locked(Server &S)
{
    std::vector<ServeJob *> ready;
    for (auto it = S.pending.begin(); it != S.pending.end();) {
        ServeJob &j = **it;
        int slot = -1;
        for (int k = 0; k < Server::kUsable[j.level] && slot < 0; ++k) {
            const int q = j.level * Server::kPerLevel + k;
            if (!S.stream_busy[q]) slot = q;
        }
        if (slot < 0) {
            ++S.stats.admission_waits;
            ++it;
            continue;
        }
        int rc = S.dev.alloc(j.dev_bytes, j.dblk);
        if (rc == 0) {
            rc = S.pin.alloc(j.off_route - j.hoff, j.hblk);
            if (rc != 0) S.dev.release(j.dblk);
        }
        if (rc == 1) {
            ++S.stats.admission_waits;
            ++it;
            continue;
        }
        if (rc != 0) {  // the arena could not grow: this job fails, the others stay queued
            j.state = 3;
            j.fail_rc = rc;
            j.fail_msg = adeco_last_error();
            j.done.store(1, std::memory_order_release);
            it = S.pending.erase(it);
            continue;
        }
        j.t0 = take_event(S);
        j.t1 = take_event(S);
        j.stream = slot;
        S.stream_busy[slot] = true;
        j.state = 1;
        S.running_jobs.push_back(&j);
        S.stats.running = (uint32_t)S.running_jobs.size();
        S.stats.max_running = std::max(S.stats.max_running, S.stats.running);
        ready.push_back(&j);
        it = S.pending.erase(it);
    }
    S.stats.queued = S.pending.size();
    S.stats.arena_bytes = S.dev.allocated;
    return ready;
}

// Enqueues an admitted job on its stream: inputs H2D, zeroed sums, the
// one-item-per-CTA deposit, the ill-conditioned tets, FP64 conversion,
// results D2H into its pinned block, then the completion host function.
static int launch_job(Server &S, ServeJob &j)
{
    adeco_session *s = S.s;
    cudaStream_t st = S.streams[j.stream];
    unsigned char *dp = j.dblk.ptr;
    // the host inputs into the pinned block (the H2D copy then runs asynchronously)
    std::memcpy(j.host(j.off_req), j.rtab.data(), j.rtab.size() * sizeof(ReqSlot));
    std::memcpy(j.host(j.off_grids), j.grids.data(), j.grids.size() * sizeof(GridDesc));
    std::memcpy(j.host(j.off_items), j.items.data(), j.items.size() * sizeof(Item));
    CUDA_TRY(cudaMemcpyAsync(dp + j.off_req, j.host(j.off_req), j.off_route - j.off_req, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemsetAsync(dp, 0, j.off_stat + 16, st));
    DepositParams P = base_params(s->tuning);
    P.items = reinterpret_cast<const Item *>(dp + j.off_items);
    P.n_items = (int)j.items.size();
    P.src_kind = SRC_LATTICE_F4;
    P.grids = reinterpret_cast<const GridDesc *>(dp + j.off_grids);
    P.src = s->lattice.p;
    P.stride_y = s->nx;
    P.stride_z = (long long)s->nx * s->ny;
    P.order = s->order;
    P.out = reinterpret_cast<unsigned long long *>(dp);
    P.counter = reinterpret_cast<int *>(dp + j.off_stat);
    P.error = P.counter + 1;
    P.route_count = reinterpret_cast<unsigned long long *>(dp + j.off_stat + 8);
    P.route = reinterpret_cast<unsigned long long *>(dp + j.off_route);
    P.route_cap = j.rcap;
    P.per_cta_items = 1;
    if (j.t0) CUDA_TRY(cudaEventRecord(j.t0, st));
    if (P.n_items > 0) {
        deposit_mixed_kernel<true><<<P.n_items, kThreads, s->dp.mixed_smem, st>>>(P);
        CUDA_TRY(cudaGetLastError());
        route_fp64_kernel<<<s->dp.sms * 2, kThreads, kRouteSmem, st>>>(P);
        CUDA_TRY(cudaGetLastError());
    }
    if (j.t1) CUDA_TRY(cudaEventRecord(j.t1, st));
    const long long total = (long long)j.cells;
    const unsigned cgrid = (unsigned)std::max<long long>(1, std::min<long long>((total + 255) / 256, s->dp.sms * 8LL));
    requests_to_f64_kernel<<<cgrid, 256, 0, st>>>(reinterpret_cast<unsigned long long *>(dp),
                                                  reinterpret_cast<const ReqSlot *>(dp + j.off_req),
                                                  (int)j.rtab.size(), total);
    CUDA_TRY(cudaGetLastError());
    if (j.eager)
        CUDA_TRY(cudaMemcpyAsync(j.host(0), dp, j.off_stat + 16, cudaMemcpyDeviceToHost, st));
    else
        CUDA_TRY(cudaMemcpyAsync(j.host(j.off_stat), dp + j.off_stat, 16, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaLaunchHostFunc(st, job_finished, &j));
    return ADECO_OK;
}

// Launches admitted jobs outside the lock; a job whose enqueue failed is
// marked failed (its stream is drained before its blocks are reused).
static void launch_ready(Server &S, std::vector<ServeJob *> &ready)
{
    for (ServeJob *j : ready) {
        const int rc = launch_job(S, *j);
        if (rc == ADECO_OK) continue;
        const std::string msg = adeco_last_error();
        cudaStreamSynchronize(S.streams[j->stream]);
        cudaGetLastError();
        std::lock_guard<std::mutex> lk(S.mu);
        S.dev.release(j->dblk);
        S.stream_busy[j->stream] = false;
        S.running_jobs.erase(std::find(S.running_jobs.begin(), S.running_jobs.end(), j));
        S.stats.running = (uint32_t)S.running_jobs.size();
        j->state = 3;
        j->fail_rc = rc;
        j->fail_msg = msg;
        j->done.store(1, std::memory_order_release);
    }
    ready.clear();
}

static void dispatcher_main(Server *S)
{
    cudaSetDevice(S->s->device);
    for (;;) {
        {
            std::unique_lock<std::mutex> lk(S->cv_mu);
            S->cv.wait_for(lk, std::chrono::milliseconds(20), [S] { return S->wake || S->stop; });
            if (S->stop) return;
            S->wake = false;
        }
        std::vector<ServeJob *> ready;
        {
            std::lock_guard<std::mutex> lk(S->mu);
            // finalize_locked erases from running_jobs: iterate over a copy
            const std::vector<ServeJob *> run = S->running_jobs;
            for (ServeJob *j : run) finalize_locked(*S, *j);
            if (!S->pending.empty()) ready = admit_locked(*S);
        }
        launch_ready(*S, ready);
        {
            std::lock_guard<std::mutex> lk(S->cv_mu);
        }
        S->cv.notify_all();  // waiters in adeco_session_wait re-check their job
    }
}

static int server_get(adeco_session *s, Server *&out)
{
    std::lock_guard<std::mutex> lk(s->server_mu);
    if (!s->server) {
        std::unique_ptr<Server> S(new Server());
        S->s = s;
        size_t free_b = 0, total_b = 0;
        CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
        S->dev.device = true;
        S->dev.budget = (size_t)(s->hbm_fraction * (double)free_b);
        S->dev.min_chunk = (size_t)1 << 30;
        S->pin.device = false;
        S->pin.budget = S->dev.budget;
        S->pin.min_chunk = (size_t)256 << 20;
        S->stats.arena_budget = S->dev.budget;
        int least = 0, greatest = 0;
        CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        for (int l = 0; l < Server::kLevels; ++l) {
            // level 0 gets the greatest priority (the most negative number)
            const int prio = greatest + (least - greatest) * l / (Server::kLevels - 1);
            for (int k = 0; k < Server::kPerLevel; ++k)
                CUDA_TRY(cudaStreamCreateWithPriority(&S->streams[l * Server::kPerLevel + k], cudaStreamNonBlocking,
                                                      prio));
        }
        double sp = 0.0;
        const int nd[3] = {s->nx, s->ny, s->nz};
        for (int a = 0; a < 3; ++a) sp += (s->bbox6[2 * a + 1] - s->bbox6[2 * a]) / (double)std::max(1, nd[a] - 1);
        S->spacing = std::max(sp / 3.0, 1e-30);
        S->dispatcher = std::thread(dispatcher_main, S.get());
        s->server = S.release();
    }
    out = s->server;
    return ADECO_OK;
}

// Work-item shape of a request grid of d cells per axis whose tets are r
// cells wide (lattice spacing over cell size): an item is (tile of T cells
// per axis, block of e^3 cubes of one meta-cell).  Expected candidate pairs
// of an item: the block's tets that reach the tile, 6 min(e, T/r + 1)^3,
// each meeting min(T, r + 1)^3 of the tile's cells.  The item target W is the
// request's expected pairs spread over 4 waves of the GPU's CTA slots, within
// [2^14, item_pairs]; of the shapes (T = the tuned edge halved down to 8,
// e = 7, 4 or 2) whose items stay under W, the one with the fewest items is
// taken (none: the smallest items).  One (tile, meta-cell) item of a 64^3
// tile held ~1e7 pairs on fine grids, and ~1e5 on tet-sized cells where a
// 128^3 request then had ~800 items: a few waves of long items whose tail
// left most of the GPU idle.
struct ItemShape {
    int tile, cubes;
};
static ItemShape request_shape(int tile, double item_pairs, int slots, int d, double r, double req_pairs)
{
    const double W = std::min(item_pairs, std::max(16384.0, req_pairs / (4.0 * slots)));
    ItemShape best{std::max(1, std::min(tile, d)), kMetaCubes};
    double best_items = -1.0, best_est = 1e300;
    bool feasible = false;
    for (int T = std::max(1, std::min(tile, d));; T = (T + 1) / 2) {
        for (int e : {kMetaCubes, 4, 2}) {
            const double reach = std::min((double)e, (double)T / r + 1.0);
            const double est = 6.0 * reach * reach * reach * std::pow(std::min((double)T, r + 1.0), 3.0);
            const double tiles = std::pow(std::ceil((double)d / T), 3.0);
            const double metas = std::pow((double)T / (kMetaCubes * r) + 1.0, 3.0);
            const double blocks = std::pow(std::ceil((double)kMetaCubes / e), 3.0);
            const double items = tiles * metas * blocks;
            if (est <= W) {
                if (!feasible || items < best_items) best = {T, e}, best_items = items;
                feasible = true;
            } else if (!feasible && est < best_est) {
                best = {T, e};
                best_est = est;
            }
        }
        if (T <= 8) break;
    }
    return best;
}

static void request_box(const adeco_request &r, float bb[6])
{
    const float h = 0.5f * r.side;
    for (int a = 0; a < 3; ++a) {
        bb[2 * a] = r.center[a] - h;
        bb[2 * a + 1] = r.center[a] + h;
    }
}

static void server_destroy(adeco_session *s)
{
    Server *S = s->server;
    if (!S) return;
    {
        std::lock_guard<std::mutex> lk(S->cv_mu);
        S->stop = true;
    }
    S->cv.notify_all();
    if (S->dispatcher.joinable()) S->dispatcher.join();
    for (cudaStream_t st : S->streams)
        if (st) {
            cudaStreamSynchronize(st);
            cudaStreamDestroy(st);
        }
    for (cudaEvent_t e : S->event_pool) cudaEventDestroy(e);
    for (auto &kv : S->jobs) {
        if (kv.second->t0) cudaEventDestroy(kv.second->t0);
        if (kv.second->t1) cudaEventDestroy(kv.second->t1);
    }
    delete S;
    s->server = nullptr;
}

extern "C" int adeco_session_get_tuning(adeco_session *s, adeco_tuning *t)
{
    if (!s || !t) return fail(ADECO_ERR_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    t->zoom_tile = s->tuning.zoom_tile;
    t->share_chunk = s->tuning.share_chunk;
    t->clip_batch = s->tuning.clip_batch;
    t->ctas_per_sm = s->tuning.ctas_per_sm > 0 ? s->tuning.ctas_per_sm : s->dp.mixed_blocks_per_sm;
    t->route_capacity = s->tuning.route_capacity;
    t->item_pairs = s->tuning.item_pairs;
    return ADECO_OK;
}

extern "C" int adeco_session_set_tuning(adeco_session *s, const adeco_tuning *t)
{
    if (!s || !t) return fail(ADECO_ERR_ARGUMENT, "null argument");
    if (t->zoom_tile < 16 || t->zoom_tile > 256) return fail(ADECO_ERR_ARGUMENT, "zoom_tile %d out of [16,256]", t->zoom_tile);
    if (t->share_chunk < 64 || t->share_chunk > 8192)
        return fail(ADECO_ERR_ARGUMENT, "share_chunk %d out of [64,8192]", t->share_chunk);
    if (t->clip_batch < 64 || t->clip_batch > kQueue)
        return fail(ADECO_ERR_ARGUMENT, "clip_batch %d out of [64,%d]", t->clip_batch, kQueue);
    if (t->ctas_per_sm < 1 || t->ctas_per_sm > 2) return fail(ADECO_ERR_ARGUMENT, "ctas_per_sm %d out of [1,2]", t->ctas_per_sm);
    if (t->item_pairs < 4096 || t->item_pairs > (1u << 26))
        return fail(ADECO_ERR_ARGUMENT, "item_pairs %u out of [4096,2^26]", t->item_pairs);
    std::lock_guard<std::mutex> lk(s->mu);
    session_drop_graph(s);  // a captured leaf replay holds the old parameters
    s->tuning.zoom_tile = t->zoom_tile;
    s->tuning.share_chunk = t->share_chunk;
    s->tuning.clip_batch = t->clip_batch;
    s->tuning.ctas_per_sm = t->ctas_per_sm;
    s->tuning.route_capacity = t->route_capacity;
    s->tuning.item_pairs = t->item_pairs;
    return ADECO_OK;
}

extern "C" int adeco_session_submit(adeco_session *s, const adeco_request *reqs, int n, uint64_t *batch_id)
{
    if (!s || !reqs || n <= 0 || !batch_id) return fail(ADECO_ERR_ARGUMENT, "bad arguments");
    for (int i = 0; i < n; ++i) {
        if (reqs[i].dims < 1 || reqs[i].dims > 1024) return fail(ADECO_ERR_ARGUMENT, "request %d: dims out of [1,1024]", i);
        if (!(reqs[i].side > 0.f)) return fail(ADECO_ERR_ARGUMENT, "request %d: side must be > 0", i);
        if (reqs[i].precision != ADECO_PREC_MIXED) return fail(ADECO_ERR_ARGUMENT, "request %d: batches run the mixed path", i);
    }
    CUDA_TRY(cudaSetDevice(s->device));
    Server *S = nullptr;
    int rc = server_get(s, S);
    if (rc) return rc;
    std::unique_ptr<ServeJob> job(new ServeJob());
    ServeJob &j = *job;
    j.srv = S;
    j.t_submit = std::chrono::steady_clock::now();
    j.reqs.assign(reqs, reqs + n);
    int tile;
    double item_pairs;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (!s->meta_index.built) s->meta_index.build(s->meta);
        tile = s->tuning.zoom_tile;
        item_pairs = (double)s->tuning.item_pairs;
    }
    std::vector<uint32_t> hits;
    long long off = 0;
    for (int i = 0; i < n; ++i) {
        float bb[6];
        request_box(reqs[i], bb);
        const int d = reqs[i].dims;
        const GridDesc g0 = make_grid(bb, d, s->tet_mass, 0, off);
        // Grids are split into tiles, one work item per (tile, meta-cell):
        // when the cells are much smaller than the tets, a meta-cell's tets
        // cover very many cells, and one item per meta-cell would leave all
        // of that to a single CTA.  The tile edge is the tuned one, halved
        // while an item's expected candidate pairs exceed item_pairs.
        const double r_cells = S->spacing / ((double)reqs[i].side / d);  // tet width in cells
        const double per_side = (double)reqs[i].side / S->spacing + (double)d;
        const double req_pairs = 6.0 * per_side * per_side * per_side;  // 6 tets per cube x (1 + r)^3 cells each
        const ItemShape shape = request_shape(tile, item_pairs, s->dp.sms * s->dp.mixed_blocks_per_sm, d, r_cells,
                                              req_pairs);
        const int tile_d = shape.tile, eb = shape.cubes;
        const int nt = (d + tile_d - 1) / tile_d;
        const size_t first_grid = j.grids.size(), first = j.items.size();
        for (int tz = 0; tz < nt; ++tz)
            for (int ty = 0; ty < nt; ++ty)
                for (int tx = 0; tx < nt; ++tx) {
                    GridDesc gt = g0;
                    const int t[3] = {tx, ty, tz};
                    for (int a = 0; a < 3; ++a) {
                        gt.tile_lo[a] = t[a] * tile_d;
                        gt.tile_hi[a] = std::min(d, (t[a] + 1) * tile_d) - 1;
                        // the tile's world box widened by a cell, inside the grid box
                        gt.cull_min[a] = std::max(g0.gmin[a], g0.gmin[a] + (float)(gt.tile_lo[a] - 1) * g0.delta[a]);
                        gt.cull_max[a] = std::min(g0.gmax[a], g0.gmin[a] + (float)(gt.tile_hi[a] + 2) * g0.delta[a]);
                    }
                    const float box6[6] = {gt.cull_min[0], gt.cull_min[1], gt.cull_min[2],
                                           gt.cull_max[0], gt.cull_max[1], gt.cull_max[2]};
                    s->meta_index.query(s->meta, box6, hits);
                    if (hits.empty()) continue;
                    const int grid_index = (int)j.grids.size();
                    j.grids.push_back(gt);
                    for (const uint32_t id : hits) {
                        int org[3], nv[3];
                        s->meta.range(id, org, nv);
                        // blocks of at most eb^3 of the meta-cell's cubes
                        for (int bz = 0; bz < nv[2] - 1; bz += eb)
                            for (int by = 0; by < nv[1] - 1; by += eb)
                                for (int bx = 0; bx < nv[0] - 1; bx += eb) {
                                    const int vx = std::min(eb, nv[0] - 1 - bx) + 1, vy = std::min(eb, nv[1] - 1 - by) + 1,
                                              vz = std::min(eb, nv[2] - 1 - bz) + 1;
                                    Item it;
                                    it.base = (org[0] + bx) + (long long)s->nx * ((org[1] + by) + (long long)s->ny * (org[2] + bz));
                                    it.grid = grid_index;
                                    it.nv = vx | (vy << 8) | (vz << 16);
                                    j.items.push_back(it);
                                }
                    }
                }
        // fixed-point scale from the tets the request can see (all its tiles)
        const int shift = choose_shift(2058.0 * (double)std::max<size_t>(1, j.items.size() - first), s->tet_mass);
        for (size_t k = first_grid; k < j.grids.size(); ++k) j.grids[k].shift = shift;
        ReqSlot r;
        std::memset(&r, 0, sizeof r);
        r.offset = off;
        r.cells = (long long)d * d * d;
        r.shift = shift;
        j.rtab.push_back(r);
        // expected candidate pairs: 6 tets per lattice cube over the box, each
        // meeting (1 + spacing / cell)^3 cells
        j.est_pairs += req_pairs;
        off += (long long)d * d * d;
    }
    j.cells = (size_t)off;
    // priority class from the expected pairs (128^3 requests over a 256^3
    // lattice in a box of 100 units: sides of 2 / 10 / 20 / 50 units take
    // about 1 / 4 / 8 / 15 ms alone on a GB300)
    j.level = j.est_pairs < kClassPairs[0] ? 0 : (j.est_pairs < kClassPairs[1] ? 1 : 2);
    // layout of the job's block
    // route list: the allocating paths' rule (an eighth of a whole meta-cell's
    // 2058 tets per item, at least 65536) counted in cubes, since a request's
    // items may hold smaller blocks
    long long cubes = 0;
    for (const Item &it : j.items)
        cubes += (long long)((it.nv & 0xff) - 1) * (((it.nv >> 8) & 0xff) - 1) * (((it.nv >> 16) & 0xff) - 1);
    unsigned long long rcap = route_capacity((cubes * 6 / 8 + 255) / 256);
    if (s->tuning.route_capacity) rcap = std::min<unsigned long long>(rcap, s->tuning.route_capacity);
    j.rcap = rcap;
    j.off_stat = round_up(j.cells * sizeof(unsigned long long), 16);
    j.eager = j.off_stat <= kEagerBytes;
    j.hoff = j.eager ? 0 : j.off_stat;
    j.off_req = round_up(j.off_stat + 16, 256);
    j.off_grids = round_up(j.off_req + j.rtab.size() * sizeof(ReqSlot), 256);
    j.off_items = round_up(j.off_grids + j.grids.size() * sizeof(GridDesc), 256);
    j.off_route = round_up(j.off_items + j.items.size() * sizeof(Item), 256);
    j.dev_bytes = round_up(j.off_route + (size_t)rcap * sizeof(unsigned long long), 256);
    if (j.dev_bytes > S->dev.budget)
        return fail(ADECO_ERR_MEMORY, "batch needs %zu bytes of device memory, admission budget %zu", j.dev_bytes,
                    S->dev.budget);
    std::vector<ServeJob *> ready;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        j.id = S->next_id++;
        *batch_id = j.id;
        S->pending.push_back(&j);
        ++S->stats.submitted;
        S->jobs[j.id] = std::move(job);
        ready = admit_locked(*S);
    }
    launch_ready(*S, ready);
    return ADECO_OK;
}

static ServeJob *find_job(adeco_session *s, uint64_t id)
{
    Server *S = s->server;
    if (!S) return nullptr;
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->jobs.find(id);
    return it == S->jobs.end() ? nullptr : it->second.get();
}

// ADECO_OK once the job's results are in its pinned block; its error status otherwise.
static int job_status(ServeJob &j, int *done)
{
    if (!j.done.load(std::memory_order_acquire)) {
        *done = 0;
        return ADECO_OK;
    }
    *done = 1;
    if (j.state == 3) return fail(j.fail_rc, "batch %llu failed: %s", (unsigned long long)j.id, j.fail_msg.c_str());
    return ADECO_OK;
}

extern "C" int adeco_session_poll(adeco_session *s, uint64_t batch_id, int *done)
{
    if (!s || !done) return fail(ADECO_ERR_ARGUMENT, "null argument");
    ServeJob *j = find_job(s, batch_id);
    if (!j) return fail(ADECO_ERR_NOT_FOUND, "unknown batch %llu", (unsigned long long)batch_id);
    return job_status(*j, done);
}

extern "C" int adeco_session_wait(adeco_session *s, uint64_t batch_id, double timeout_s)
{
    if (!s) return fail(ADECO_ERR_ARGUMENT, "null session");
    ServeJob *j = find_job(s, batch_id);
    if (!j) return fail(ADECO_ERR_NOT_FOUND, "unknown batch %llu", (unsigned long long)batch_id);
    Server *S = s->server;
    const auto deadline = std::chrono::steady_clock::now() + std::chrono::duration<double>(timeout_s);
    std::unique_lock<std::mutex> lk(S->cv_mu);
    while (!j->done.load(std::memory_order_acquire)) {
        if (std::chrono::steady_clock::now() > deadline)
            return fail(ADECO_ERR_STATE, "timed out after %.1f s waiting for batch %llu", timeout_s,
                        (unsigned long long)batch_id);
        S->cv.wait_for(lk, std::chrono::milliseconds(5));
    }
    lk.unlock();
    int done = 0;
    return job_status(*j, &done);
}

// The finished job's device error flag (finalising it if the dispatcher has not yet).
static int job_error(adeco_session *s, ServeJob &j)
{
    Server *S = s->server;
    std::lock_guard<std::mutex> lk(S->mu);
    finalize_locked(*S, j);
    return j.err_bits;
}

extern "C" int adeco_session_result(adeco_session *s, uint64_t batch_id, int index, double *host_out, size_t capacity)
{
    if (!s || !host_out) return fail(ADECO_ERR_ARGUMENT, "null argument");
    ServeJob *j = find_job(s, batch_id);
    if (!j) return fail(ADECO_ERR_NOT_FOUND, "unknown batch %llu", (unsigned long long)batch_id);
    if (index < 0 || index >= (int)j->reqs.size()) return fail(ADECO_ERR_ARGUMENT, "request index out of range");
    int rc = adeco_session_wait(s, batch_id, 3600.0);
    if (rc) return rc;
    const int err = job_error(s, *j);
    if (err) return deposit_error(err, "a zoom grid");
    const size_t n = (size_t)j->rtab[index].cells;
    if (capacity < n) return fail(ADECO_ERR_ARGUMENT, "capacity %zu < %zu cells", capacity, n);
    const size_t off = (size_t)j->rtab[index].offset * sizeof(double);
    if (j->eager) {
        std::memcpy(host_out, j->host(off), n * sizeof(double));
    } else {
        CUDA_TRY(cudaSetDevice(s->device));
        CUDA_TRY(cudaMemcpy(host_out, j->dblk.ptr + off, n * sizeof(double), cudaMemcpyDeviceToHost));
    }
    return ADECO_OK;
}

extern "C" int adeco_session_latency(adeco_session *s, uint64_t batch_id, int index, double *ms)
{
    if (!s || !ms) return fail(ADECO_ERR_ARGUMENT, "null argument");
    ServeJob *j = find_job(s, batch_id);
    if (!j) return fail(ADECO_ERR_NOT_FOUND, "unknown batch %llu", (unsigned long long)batch_id);
    if (index < 0 || index >= (int)j->reqs.size()) return fail(ADECO_ERR_ARGUMENT, "request index out of range");
    if (!j->done.load(std::memory_order_acquire)) return fail(ADECO_ERR_STATE, "batch not finished");
    *ms = std::chrono::duration<double, std::milli>(j->t_done - j->t_submit).count();
    return ADECO_OK;
}

extern "C" int adeco_session_batch_device_ms(adeco_session *s, uint64_t batch_id, double *ms)
{
    if (!s || !ms) return fail(ADECO_ERR_ARGUMENT, "null argument");
    ServeJob *j = find_job(s, batch_id);
    if (!j) return fail(ADECO_ERR_NOT_FOUND, "unknown batch %llu", (unsigned long long)batch_id);
    int rc = adeco_session_wait(s, batch_id, 3600.0);
    if (rc) return rc;
    if (!j->t0 || !j->t1) return fail(ADECO_ERR_STATE, "no timing events for batch %llu", (unsigned long long)batch_id);
    float f = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&f, j->t0, j->t1));
    *ms = f;
    return ADECO_OK;
}

extern "C" int adeco_session_release(adeco_session *s, uint64_t batch_id)
{
    if (!s) return fail(ADECO_ERR_ARGUMENT, "null session");
    Server *S = s->server;
    if (!S || !find_job(s, batch_id)) return fail(ADECO_ERR_NOT_FOUND, "unknown batch");
    // a batch still queued or running is waited for (on the host: no device synchronisation)
    const int wrc = adeco_session_wait(s, batch_id, 3600.0);
    if (wrc == ADECO_ERR_STATE) return wrc;
    std::unique_ptr<ServeJob> j;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        auto it = S->jobs.find(batch_id);
        if (it == S->jobs.end()) return fail(ADECO_ERR_NOT_FOUND, "unknown batch");
        ServeJob &jr = *it->second;
        finalize_locked(*S, jr);
        S->pin.release(jr.hblk);
        if (!jr.eager) S->dev.release(jr.dblk);
        if (jr.t0) S->event_pool.push_back(jr.t0);
        if (jr.t1) S->event_pool.push_back(jr.t1);
        jr.t0 = jr.t1 = nullptr;
        j = std::move(it->second);
        S->jobs.erase(it);
    }
    S->signal();  // its pinned block may let a queued batch in
    return ADECO_OK;
}

extern "C" int adeco_session_serving_stats(adeco_session *s, adeco_serving_stats *st)
{
    if (!s || !st) return fail(ADECO_ERR_ARGUMENT, "null argument");
    Server *S = s->server;
    if (!S) {
        std::memset(st, 0, sizeof *st);
        return ADECO_OK;
    }
    std::lock_guard<std::mutex> lk(S->mu);
    *st = S->stats;
    st->queued = S->pending.size();
    st->arena_bytes = S->dev.allocated;
    return ADECO_OK;
}
