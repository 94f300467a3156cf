// runtime.cu -- host runtime and C ABI of libadeco_gb300.so (include/adeco_deposit.h).
//
// One process drives one GPU.  The reference boundary (adeco_deposit_tets*)
// replaces DepositWrapper::deposit_tets / resample() (src/AdDeposit2Grid.cu:229-584):
// positions are copied to HBM once per call, the deposit runs as one
// persistent launch over (grid, vertex-block) work items, and the result is
// added into the caller's grid.  Sessions keep the particle lattice, its
// meta-cells and the octree resident and run the leaf deposit either as one
// batched persistent launch (mixed precision) or as one FP64 launch per leaf
// (the plain baseline).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/adeco_deposit.h"
#include "kernels.cuh"
#include "octree.h"

using namespace adeco;

// ------------------------------------------------------------- errors
static thread_local std::string g_last_error;

static int fail(int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

#define CUDA_TRY(call)                                                                                   \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess) return fail(ADECO_ERR_CUDA, "%s failed: %s (%s:%d)", #call,               \
                                           cudaGetErrorString(e_), __FILE__, __LINE__);                  \
    } while (0)

extern "C" const char *adeco_last_error(void) { return g_last_error.c_str(); }
extern "C" int adeco_abi_version(void) { return ADECO_ABI_VERSION; }

// ------------------------------------------------------------- helpers
namespace {

template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    ~DevBuf() { release(); }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    int reserve(size_t count)
    {
        if (count <= n && p) return ADECO_OK;
        release();
        if (count == 0) count = 1;
        cudaError_t e = cudaMalloc(&p, count * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            return fail(e == cudaErrorMemoryAllocation ? ADECO_ERR_MEMORY : ADECO_ERR_CUDA,
                        "cudaMalloc of %zu bytes failed: %s", count * sizeof(T), cudaGetErrorString(e));
        }
        n = count;
        return ADECO_OK;
    }
};

// fixed-point exponent for a grid that at most `tets` tets of mass `mass` touch
int choose_shift(double tets, double mass)
{
    const double bound = std::max(tets * std::max(mass, 1e-30), 1e-30);
    int s = 62 - (int)std::ceil(std::log2(bound + 1.0));
    return std::min(52, std::max(8, s));
}

// The request grid: FP32 fields reproduce the reference's range arithmetic,
// FP64 fields the FP64 oracle's geometry (cubic cells: scale = 1/dx on all
// axes, as src/AdDepositTets2Grid.h:569).
GridDesc make_grid(const float bbox[6], int dims, double tet_mass, int shift, long long out_offset)
{
    GridDesc g;
    std::memset(&g, 0, sizeof g);
    for (int a = 0; a < 3; ++a) {
        g.gmin[a] = bbox[2 * a];
        g.gmax[a] = bbox[2 * a + 1];
        g.delta[a] = (g.gmax[a] - g.gmin[a]) / (float)dims;
        g.gmin_d[a] = (double)g.gmin[a];
        g.delta_d[a] = ((double)g.gmax[a] - (double)g.gmin[a]) / (double)dims;
    }
    const double s = 1.0 / g.delta_d[0];
    for (int a = 0; a < 3; ++a) g.scale_d[a] = s;
    const double cell_vol = g.delta_d[0] * g.delta_d[1] * g.delta_d[2];
    g.mass_factor = tet_mass * cell_vol * s * s * s;
    for (int a = 0; a < 3; ++a) {
        g.rcell[a] = g.delta_d[a] * g.scale_d[a];
        g.inv_rcell[a] = 1.0 / g.rcell[a];
        g.drcell[a] = (float)(g.rcell[a] - 1.0);
        g.inv_rcell_f[a] = (float)g.inv_rcell[a];
    }
    g.tet_mass = (float)tet_mass;
    for (int a = 0; a < 3; ++a) {
        g.scale_hi[a] = (float)g.scale_d[a];
        g.scale_lo[a] = (float)(g.scale_d[a] - (double)g.scale_hi[a]);
    }
    g.mf_hi = (float)g.mass_factor;
    g.mf_lo = (float)(g.mass_factor - (double)g.mf_hi);
    g.dims = dims;
    g.shift = shift;
    g.out_offset = out_offset;
    for (int a = 0; a < 3; ++a) {
        g.tile_lo[a] = 0;
        g.tile_hi[a] = dims - 1;
        g.cull_min[a] = g.gmin[a];
        g.cull_max[a] = g.gmax[a];
    }
    return g;
}

struct DeviceProps {
    int sms = 0;
    int mixed_blocks_per_sm = 0;
    size_t mixed_smem = 0;
};

int mixed_setup(int device, DeviceProps &dp)
{
    static std::mutex mu;
    static std::map<int, DeviceProps> cache;
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(device);
    if (it != cache.end()) {
        dp = it->second;
        return ADECO_OK;
    }
    cudaDeviceProp prop;
    CUDA_TRY(cudaGetDeviceProperties(&prop, device));
    dp.sms = prop.multiProcessorCount;
    dp.mixed_smem = sizeof(SharedMixed);
    CUDA_TRY(cudaFuncSetAttribute(deposit_mixed_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)dp.mixed_smem));
    CUDA_TRY(cudaFuncSetAttribute(deposit_mixed_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)dp.mixed_smem));
    CUDA_TRY(cudaFuncSetAttribute(route_fp64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRouteSmem));
    int nb = 0;
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, deposit_mixed_kernel<false>, kThreads, dp.mixed_smem));
    dp.mixed_blocks_per_sm = std::max(1, nb);
    cache[device] = dp;
    return ADECO_OK;
}

// Launch-shape and batching parameters (adeco_tuning), per session.
struct Tuning {
    int zoom_tile = 64;                       // cells per tile edge of a zoom grid
    int share_chunk = kChunk;                 // work sharing: pairs per chunk
    int clip_batch = kQueue;                  // partial pairs listed per warp before clipping
    int ctas_per_sm = 0;                      // persistent launches: CTAs per SM (0: occupancy)
    unsigned long long route_capacity = 0;    // 0: route_capacity(items)
    unsigned item_pairs = 1u << 18;           // zoom grids: expected candidate pairs per work item
};

// Deposit parameters with every field that is not a pointer or a count set
// to its default (or tuned) value.
DepositParams base_params(const Tuning &t)
{
    DepositParams P;
    std::memset(&P, 0, sizeof P);
    P.per_cta_items = 0;
    P.share_chunk = t.share_chunk;
    P.clip_batch = t.clip_batch;
    P.help_spins = kHelpSpins;
    P.close_spins = kCloseSpins;
    return P;
}

// Entries of the list of ill-conditioned tets a mixed launch over n_items
// items may fill (count word + entries; 8 bytes each): a quarter of a tet per
// item on average, at least 64K, at most 64M.
static constexpr unsigned long long route_capacity(long long n_items)
{
    return (unsigned long long)std::min<long long>(1LL << 26, std::max<long long>(65536, n_items * 256));
}

// Points P at a route list buffer of route_capacity(...) + 1 words.
static void set_route(DepositParams &P, unsigned long long *buf, unsigned long long cap)
{
    P.route_count = buf;
    P.route = buf + 1;
    P.route_cap = cap;
}

// Message for the device error flag of a mixed launch.
static int deposit_error(int err, const char *where)
{
    if (err & 4) return fail(ADECO_ERR_LIMIT, "more ill-conditioned tets in %s than the route list holds", where);
    if (err & 8) return fail(ADECO_ERR_CUDA, "a warp of %s timed out waiting for the warps sharing its pairs", where);
    return fail(ADECO_ERR_LIMIT, "a tet spans more than 2^25 candidate cells of %s", where);
}

// One persistent launch of the mixed kernel over `n_items` items, then the
// launch that deposits the ill-conditioned tets it listed.  share: warps of
// an item share the pairs of large tet groups (zoom grids, whose cells are
// much smaller than the tets).
int launch_mixed(const DeviceProps &dp, DepositParams P, bool share, cudaStream_t st, int ctas_per_sm = 0)
{
    if (P.n_items <= 0) return ADECO_OK;
    CUDA_TRY(cudaMemsetAsync(P.counter, 0, sizeof(int), st));
    CUDA_TRY(cudaMemsetAsync(P.route_count, 0, sizeof(unsigned long long), st));
    const int per_sm = ctas_per_sm > 0 ? std::min(ctas_per_sm, dp.mixed_blocks_per_sm) : dp.mixed_blocks_per_sm;
    const int grid = std::max(1, std::min(P.n_items, dp.sms * per_sm));
    if (share)
        deposit_mixed_kernel<true><<<grid, kThreads, dp.mixed_smem, st>>>(P);
    else
        deposit_mixed_kernel<false><<<grid, kThreads, dp.mixed_smem, st>>>(P);
    CUDA_TRY(cudaGetLastError());
    route_fp64_kernel<<<dp.sms * 2, kThreads, kRouteSmem, st>>>(P);  // the resident CTAs
    CUDA_TRY(cudaGetLastError());
    return ADECO_OK;
}

// Plain FP64 launch over the cubes of `n_items` items.
// d_cube_off: n_items+1 cube offsets of the items (device), [c0, c1) their range.
int launch_plain(const DeviceProps &dp, DepositParams P, const long long *d_cube_off, long long c0, long long c1,
                 cudaStream_t st)
{
    if (P.n_items <= 0 || c1 <= c0) return ADECO_OK;
    const long long warps = c1 - c0;
    const long long want = (warps * 32 + kThreads - 1) / kThreads;
    const int grid = (int)std::max(1LL, std::min(want, (long long)dp.sms * 8));
    deposit_plain_fp64_kernel<<<grid, kThreads, 0, st>>>(P, c0, c1, d_cube_off);
    CUDA_TRY(cudaGetLastError());
    return ADECO_OK;
}

int select_device(int use_specific_gpu, size_t device_id, int &dev)
{
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count <= 0)
        return fail(ADECO_ERR_DEVICE, "no CUDA device available (%s)", cudaGetErrorString(e));
    if (use_specific_gpu && device_id >= (size_t)count)
        return fail(ADECO_ERR_DEVICE, "selected invalid device number: %zu of %d devices", device_id, count);
    dev = use_specific_gpu ? (int)device_id : 0;
    CUDA_TRY(cudaSetDevice(dev));
    return ADECO_OK;
}

// Work items for patches [p0, p0+np) of (m+1)^3-vertex patches: sub-blocks of
// at most 7^3 cubes each.
void patch_items(size_t p0, size_t np, int m, int grid, std::vector<Item> &items, std::vector<long long> *cube_off)
{
    const long long n1 = m + 1, n2 = n1 * n1;
    const int nsb = MetaGrid::ceil_div(m, kMetaCubes);
    long long cubes = cube_off && !cube_off->empty() ? cube_off->back() : 0;
    for (size_t p = p0; p < p0 + np; ++p) {
        const long long pbase = (long long)p * n1 * n2;
        for (int sz = 0; sz < nsb; ++sz)
            for (int sy = 0; sy < nsb; ++sy)
                for (int sx = 0; sx < nsb; ++sx) {
                    const int ox = sx * kMetaCubes, oy = sy * kMetaCubes, oz = sz * kMetaCubes;
                    const int vx = std::min(kMetaCubes + 1, m + 1 - ox), vy = std::min(kMetaCubes + 1, m + 1 - oy),
                              vz = std::min(kMetaCubes + 1, m + 1 - oz);
                    Item it;
                    it.base = pbase + ox + n1 * oy + n2 * oz;
                    it.grid = grid;
                    it.nv = vx | (vy << 8) | (vz << 16);
                    items.push_back(it);
                    if (cube_off) {
                        cube_off->push_back(cubes);
                        cubes += (long long)(vx - 1) * (vy - 1) * (vz - 1);
                    }
                }
    }
    if (cube_off) cube_off->push_back(cubes);
}

int validate_boundary(size_t patch_offset, size_t num_patches, const float *positions, size_t positions_size, int m,
                      const float *bbox, int dims, const void *data)
{
    if (m < 1) return fail(ADECO_ERR_ARGUMENT, "meta_cells_per_patch must be >= 1 (got %d)", m);
    if (dims < 1) return fail(ADECO_ERR_ARGUMENT, "dims must be >= 1 (got %d)", dims);
    if (dims > 4096) return fail(ADECO_ERR_LIMIT, "dims %d above the supported 4096", dims);
    if (!positions || !bbox || !data) return fail(ADECO_ERR_ARGUMENT, "null positions, bbox or data pointer");
    const size_t fpp = 3 * (size_t)(m + 1) * (m + 1) * (m + 1);
    const size_t cpp = (size_t)m * m * m;
    if (num_patches * cpp >= (size_t)INT_MAX)
        return fail(ADECO_ERR_OVERFLOW, "num_cells will cause integer overflow (%zu patches of %zu cubes)",
                    num_patches, cpp);
    if (positions_size % fpp != 0)
        return fail(ADECO_ERR_ARGUMENT, "positions_size %zu is not a multiple of %zu floats per patch",
                    positions_size, fpp);
    if (patch_offset + num_patches > positions_size / fpp)
        return fail(ADECO_ERR_INCONSISTENT, "inconsistent point array: patches [%zu,%zu) of %zu", patch_offset,
                    patch_offset + num_patches, positions_size / fpp);
    for (int a = 0; a < 3; ++a)
        if (!(bbox[2 * a + 1] > bbox[2 * a]))
            return fail(ADECO_ERR_ARGUMENT, "bbox axis %d is empty (%g >= %g)", a, bbox[2 * a], bbox[2 * a + 1]);
    return ADECO_OK;
}

}  // namespace

// ============================================================ boundary
// Per-thread workspace of the boundary entry points.  The reference's
// deposit_tets is called from several pthreads at once, one grid each
// (src/AdDynamicLoadBalancing.h:200-205), and allocates and frees its device
// memory and stream on every call (src/AdDeposit2Grid.cu:353-394, 527-534);
// here each thread's buffers grow to its largest call and are kept, so a
// repeated call makes no cudaMalloc, cudaFree (which synchronises the device)
// or stream creation.  Freed when the thread exits.
namespace {
struct BoundaryWork {
    int dev = -1;
    cudaStream_t stream = nullptr;  // the reference-signature calls' stream
    DevBuf<Item> items;
    DevBuf<GridDesc> grid;
    DevBuf<int> counter;
    DevBuf<long long> cube_off;
    DevBuf<unsigned long long> route, fixed;
    DevBuf<double> f64, packed;
    DevBuf<float> pos, part;
    double *pinned = nullptr;  // D2H staging of the grid
    size_t pinned_n = 0;
    float *pin_part = nullptr;  // D2H staging of the vertex-box partials
    ~BoundaryWork() { drop(); }
    void drop()
    {
        items.release(); grid.release(); counter.release(); cube_off.release();
        route.release(); fixed.release(); f64.release(); packed.release(); pos.release(); part.release();
        if (pinned) cudaFreeHost(pinned);
        pinned = nullptr;
        pinned_n = 0;
        if (pin_part) cudaFreeHost(pin_part);
        pin_part = nullptr;
        if (stream) cudaStreamDestroy(stream);
        stream = nullptr;
    }
    // the current device's workspace (a thread that moves to another device starts afresh)
    int bind(int device)
    {
        if (dev == device) return ADECO_OK;
        drop();
        dev = device;
        CUDA_TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        return ADECO_OK;
    }
    int box_staging()
    {
        if (pin_part) return ADECO_OK;
        if (int rc = part.reserve(kBoxBlocks * 7)) return rc;
        CUDA_TRY(cudaHostAlloc((void **)&pin_part, kBoxBlocks * 7 * sizeof(float), cudaHostAllocDefault));
        return ADECO_OK;
    }
    static constexpr int kBoxBlocks = 256;
    int staging(size_t n)
    {
        if (n <= pinned_n) return ADECO_OK;
        if (pinned) cudaFreeHost(pinned);
        pinned = nullptr;
        pinned_n = 0;
        CUDA_TRY(cudaHostAlloc((void **)&pinned, n * sizeof(double), cudaHostAllocDefault));
        pinned_n = n;
        return ADECO_OK;
    }
};
thread_local BoundaryWork t_work;
}  // namespace

// Deposit patches [patch_offset, +num_patches) of device-resident patch data
// into d_fixed (mixed, fixed point 2^shift) or d_f64 (plain FP64).
static int deposit_device_core(int dev, const float *d_pos, size_t patch_offset, size_t num_patches, int m,
                               const float *bbox, int dims, int precision, int order, double tet_mass,
                               unsigned long long *d_fixed, double *d_f64, int shift, cudaStream_t st)
{
    DeviceProps dp;
    int rc = mixed_setup(dev, dp);
    if (rc) return rc;
    std::vector<Item> items;
    std::vector<long long> cube_off;
    patch_items(patch_offset, num_patches, m, 0, items, precision == ADECO_PREC_FP64 ? &cube_off : nullptr);
    GridDesc g = make_grid(bbox, dims, tet_mass, shift, 0);
    if ((rc = t_work.bind(dev))) return rc;
    DevBuf<Item> &d_items = t_work.items;
    DevBuf<GridDesc> &d_grid = t_work.grid;
    DevBuf<int> &d_counter = t_work.counter;
    DevBuf<long long> &d_cube_off = t_work.cube_off;
    DevBuf<unsigned long long> &d_route = t_work.route;
    const unsigned long long rcap = route_capacity((long long)items.size());
    if ((rc = d_items.reserve(items.size())) || (rc = d_grid.reserve(1)) || (rc = d_counter.reserve(2))) return rc;
    if (precision != ADECO_PREC_FP64 && (rc = d_route.reserve(rcap + 1))) return rc;
    CUDA_TRY(cudaMemsetAsync(d_counter.p, 0, 2 * sizeof(int), st));
    CUDA_TRY(cudaMemcpyAsync(d_items.p, items.data(), items.size() * sizeof(Item), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_grid.p, &g, sizeof g, cudaMemcpyHostToDevice, st));
    DepositParams P = base_params(Tuning());
    P.items = d_items.p;
    P.n_items = (int)items.size();
    P.src_kind = SRC_PATCH_F3;
    P.grids = d_grid.p;
    P.src = d_pos;
    P.stride_y = m + 1;
    P.stride_z = (long long)(m + 1) * (m + 1);
    P.order = order;
    P.pad_check = 1;
    P.out = d_fixed;
    P.out_d = d_f64;
    P.counter = d_counter.p;
    P.error = d_counter.p + 1;
    if (precision != ADECO_PREC_FP64) set_route(P, d_route.p, rcap);
    if (precision == ADECO_PREC_FP64) {
        if ((rc = d_cube_off.reserve(cube_off.size()))) return rc;
        CUDA_TRY(cudaMemcpyAsync(d_cube_off.p, cube_off.data(), cube_off.size() * sizeof(long long),
                                 cudaMemcpyHostToDevice, st));
        rc = launch_plain(dp, P, d_cube_off.p, 0, cube_off.back(), st);
    } else {
        rc = launch_mixed(dp, P, false, st);
    }
    if (rc) return rc;
    int err = 0;
    CUDA_TRY(cudaMemcpyAsync(&err, d_counter.p + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (err) return deposit_error(err, "the grid");
    return ADECO_OK;
}

extern "C" int adeco_deposit_tets_ex(const adeco_deposit_args *a)
{
    if (!a) return fail(ADECO_ERR_ARGUMENT, "null args");
    if (a->positions_size == 0 || a->num_patches == 0) return ADECO_OK;  // the reference returns silently
    int rc = validate_boundary(a->patch_offset, a->num_patches, a->positions, a->positions_size,
                               a->meta_cells_per_patch, a->bbox, a->dims, a->data);
    if (rc) return rc;
    if (a->precision != ADECO_PREC_MIXED && a->precision != ADECO_PREC_FP64)
        return fail(ADECO_ERR_ARGUMENT, "unknown precision %d", a->precision);
    if (a->tet_order != ADECO_ORDER_REF && a->tet_order != ADECO_ORDER_CONFORMING)
        return fail(ADECO_ERR_ARGUMENT, "unknown tet order %d", a->tet_order);
    if (a->out_type != ADECO_OUT_F32 && a->out_type != ADECO_OUT_F64)
        return fail(ADECO_ERR_ARGUMENT, "unknown output type %d", a->out_type);
    int dev = 0;
    if ((rc = select_device(a->use_specific_gpu, a->device_id, dev))) return rc;
    const int m = a->meta_cells_per_patch;
    const size_t fpp = 3 * (size_t)(m + 1) * (m + 1) * (m + 1);
    const size_t ncell = (size_t)a->dims * a->dims * a->dims;
    // admission: positions slice + accumulators within 75% of free HBM (the
    // reference's MAX_GPU_USAGE); larger inputs run in several passes
    size_t free_b = 0, total_b = 0;
    CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    const size_t grid_bytes = ncell * (sizeof(unsigned long long) + sizeof(double));
    const double budget = 0.75 * (double)free_b;
    if ((double)grid_bytes >= budget)
        return fail(ADECO_ERR_MEMORY, "grid too large for device memory (%zu bytes, budget %.0f)", grid_bytes, budget);
    const size_t patch_bytes = fpp * sizeof(float);
    size_t per_pass = (size_t)((budget - (double)grid_bytes) / (double)patch_bytes);
    per_pass = std::max<size_t>(1, std::min(per_pass, a->num_patches));

    if ((rc = t_work.bind(dev))) return rc;
    cudaStream_t st = t_work.stream;
    DevBuf<float> &d_pos = t_work.pos;
    DevBuf<unsigned long long> &d_fixed = t_work.fixed;
    DevBuf<double> &d_f64 = t_work.f64;
    rc = d_pos.reserve(per_pass * fpp);
    if (!rc) rc = (a->precision == ADECO_PREC_FP64) ? d_f64.reserve(ncell) : d_fixed.reserve(ncell);
    if (!rc && a->precision == ADECO_PREC_FP64) {
        if (cudaMemsetAsync(d_f64.p, 0, ncell * sizeof(double), st) != cudaSuccess) rc = fail(ADECO_ERR_CUDA, "memset");
    } else if (!rc) {
        if (cudaMemsetAsync(d_fixed.p, 0, ncell * sizeof(unsigned long long), st) != cudaSuccess)
            rc = fail(ADECO_ERR_CUDA, "memset");
    }
    // the fixed-point scale is fixed for the whole call
    const int call_shift = choose_shift(6.0 * (double)a->num_patches * (double)m * m * m, a->tet_mass);
    // the box of the deposited vertices (padding left out), over all passes:
    // only the grid cells in its range can receive mass, so only those are
    // brought back and added (an image box of a periodic volume touches a
    // thin slab of the grid)
    float vmin[3] = {INFINITY, INFINITY, INFINITY}, vmax[3] = {-INFINITY, -INFINITY, -INFINITY};
    bool vnan = false;
    if (!rc) rc = t_work.box_staging();
    for (size_t done = 0; !rc && done < a->num_patches; done += per_pass) {
        const size_t np = std::min(per_pass, a->num_patches - done);
        const float *src = a->positions + (a->patch_offset + done) * fpp;
        if (cudaMemcpyAsync(d_pos.p, src, np * fpp * sizeof(float), cudaMemcpyHostToDevice, st) != cudaSuccess) {
            rc = fail(ADECO_ERR_CUDA, "H2D positions");
            break;
        }
        const long long nvert = (long long)(np * fpp / 3);
        const int bb_blocks = (int)std::min<long long>(BoundaryWork::kBoxBlocks, (nvert + kBoxThreads - 1) / kBoxThreads);
        patch_bbox_kernel<<<bb_blocks, kBoxThreads, 0, st>>>(d_pos.p, nvert, t_work.part.p);
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpyAsync(t_work.pin_part, t_work.part.p, (size_t)bb_blocks * 7 * sizeof(float), cudaMemcpyDeviceToHost,
                            st) != cudaSuccess) {
            rc = fail(ADECO_ERR_CUDA, "vertex box");
            break;
        }
        // every pass uses the call's shift: deposit patches [0, np) of the slice
        rc = deposit_device_core(dev, d_pos.p, 0, np, m, a->bbox, a->dims, a->precision, a->tet_order, a->tet_mass,
                                 d_fixed.p, d_f64.p, call_shift, st);
        if (rc) break;  // deposit_device_core synchronised the stream: the partials are in
        for (int b = 0; b < bb_blocks; ++b) {
            const float *q = t_work.pin_part + 7 * b;
            for (int x = 0; x < 3; ++x) {
                vmin[x] = std::fmin(vmin[x], q[x]);
                vmax[x] = std::fmax(vmax[x], q[3 + x]);
            }
            vnan = vnan || q[6] != 0.f;
        }
    }
    // the cell range of the vertex box (one cell of margin against the
    // rounding of the kernels' FP32 range arithmetic); a NaN coordinate
    // falls back to the whole grid
    int lo[3] = {0, 0, 0}, ext[3] = {a->dims, a->dims, a->dims};
    bool empty = false;
    if (!rc && !vnan) {
        for (int x = 0; x < 3; ++x) {
            const double gmin = a->bbox[2 * x], gmax = a->bbox[2 * x + 1];
            const double delta = (double)((a->bbox[2 * x + 1] - a->bbox[2 * x]) / (float)a->dims);
            if (!(vmin[x] <= vmax[x]) || (double)vmax[x] < gmin || (double)vmin[x] > gmax || !(delta > 0.0)) {
                empty = true;
                break;
            }
            const double flo = std::floor((std::fmax((double)vmin[x], gmin) - gmin) / delta) - 1.0;
            const double fhi = std::ceil((std::fmin((double)vmax[x], gmax) - gmin) / delta) + 1.0;
            const int l = (int)std::fmin(std::fmax(flo, 0.0), (double)(a->dims - 1));
            const int h = (int)std::fmin(std::fmax(fhi, 0.0), (double)(a->dims - 1));
            lo[x] = l;
            ext[x] = h - l + 1;
        }
    }
    // convert the box's cells to FP64 packed, bring them back, add them into
    // the caller's grid
    if (!rc && !empty) {
        const size_t nbox = (size_t)ext[0] * ext[1] * ext[2];
        const bool whole = nbox == ncell;
        const double *dsrc = nullptr;  // device FP64 of the box, packed
        if (a->precision == ADECO_PREC_FP64 && whole) {
            dsrc = d_f64.p;  // the plain FP64 path accumulates in FP64: the grid itself
        } else {
            DevBuf<double> &dst = (a->precision == ADECO_PREC_FP64) ? t_work.packed : d_f64;
            if ((rc = dst.reserve(nbox)) == ADECO_OK) {
                const unsigned blocks = (unsigned)std::min<size_t>(1024, (nbox + 255) / 256);
                grid_box_kernel<<<blocks, 256, 0, st>>>(a->precision == ADECO_PREC_FP64 ? nullptr : d_fixed.p, d_f64.p,
                                                        dst.p, a->dims, lo[0], lo[1], lo[2], ext[0], ext[1], ext[2],
                                                        std::ldexp(1.0, -call_shift));
                dsrc = dst.p;
            }
        }
        if (!rc) rc = t_work.staging(nbox);
        if (!rc) {
            const double *host = t_work.pinned;
            if (cudaGetLastError() != cudaSuccess ||
                cudaMemcpyAsync(t_work.pinned, dsrc, nbox * sizeof(double), cudaMemcpyDeviceToHost, st) !=
                    cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess) {
                rc = fail(ADECO_ERR_CUDA, "D2H grid: %s", cudaGetErrorString(cudaGetLastError()));
            } else {
                const size_t d = (size_t)a->dims;
                for (int z = 0; z < ext[2]; ++z)
                    for (int y = 0; y < ext[1]; ++y) {
                        const double *row = host + (size_t)ext[0] * (y + (size_t)ext[1] * z);
                        const size_t c0 = (size_t)lo[0] + d * ((size_t)(lo[1] + y) + d * (size_t)(lo[2] + z));
                        if (a->out_type == ADECO_OUT_F64) {
                            double *out = (double *)a->data + c0;
                            for (int x = 0; x < ext[0]; ++x) out[x] += row[x];
                        } else {
                            float *out = (float *)a->data + c0;
                            for (int x = 0; x < ext[0]; ++x) out[x] += (float)row[x];
                        }
                    }
            }
        }
    }
    cudaStreamSynchronize(st);
    return rc;
}

extern "C" int adeco_deposit_tets(int use_specific_gpu, size_t device_id, size_t patch_offset, size_t num_patches,
                                  const float *positions, size_t positions_size, int meta_cells_per_patch,
                                  const float bbox[6], int dims, float *data)
{
    adeco_deposit_args a;
    std::memset(&a, 0, sizeof a);
    a.use_specific_gpu = use_specific_gpu;
    a.device_id = device_id;
    a.patch_offset = patch_offset;
    a.num_patches = num_patches;
    a.positions = positions;
    a.positions_size = positions_size;
    a.meta_cells_per_patch = meta_cells_per_patch;
    a.bbox = bbox;
    a.dims = dims;
    a.data = data;
    a.out_type = ADECO_OUT_F32;
    a.precision = ADECO_PREC_MIXED;
    a.tet_order = ADECO_ORDER_REF;
    a.tet_mass = 1.0;
    return adeco_deposit_tets_ex(&a);
}

extern "C" int adeco_deposit_tets_device(const float *d_positions, size_t positions_size, size_t patch_offset,
                                         size_t num_patches, int m, const float bbox[6], int dims, double *d_out,
                                         int precision, int tet_order, double tet_mass, void *stream)
{
    if (positions_size == 0 || num_patches == 0) return ADECO_OK;
    int rc = validate_boundary(patch_offset, num_patches, d_positions, positions_size, m, bbox, dims, d_out);
    if (rc) return rc;
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    cudaStream_t st = (cudaStream_t)stream;
    const size_t ncell = (size_t)dims * dims * dims;
    const int shift = choose_shift(6.0 * (double)num_patches * (double)m * m * m, tet_mass);
    if (precision == ADECO_PREC_FP64) {
        return deposit_device_core(dev, d_positions, patch_offset, num_patches, m, bbox, dims, precision, tet_order,
                                   tet_mass, nullptr, d_out, shift, st);
    }
    if ((rc = t_work.bind(dev))) return rc;
    DevBuf<unsigned long long> &d_fixed = t_work.fixed;
    if ((rc = d_fixed.reserve(ncell))) return rc;
    CUDA_TRY(cudaMemsetAsync(d_fixed.p, 0, ncell * sizeof(unsigned long long), st));
    rc = deposit_device_core(dev, d_positions, patch_offset, num_patches, m, bbox, dims, precision, tet_order,
                             tet_mass, d_fixed.p, nullptr, shift, st);
    if (rc) return rc;
    fixed_accumulate_f64_kernel<<<1024, 256, 0, st>>>(d_fixed.p, d_out, (long long)ncell, std::ldexp(1.0, -shift));
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(st));
    return ADECO_OK;
}

// ============================================================ sessions
struct adeco_session {
    int device = 0;
    int order = ORDER_REF;
    double tet_mass = 1.0;
    double hbm_fraction = 0.75;
    int acc_fp64 = 1;
    cudaStream_t stream = nullptr;
    DeviceProps dp;
    int nx = 0, ny = 0, nz = 0;
    DevBuf<float4> lattice;
    MetaGrid meta;
    DevBuf<float> d_meta_bbox;  // the meta-cells' AABBs, also on the device (octree builder)
    int octree_builder = ADECO_OCTREE_DEVICE;
    MetaIndex meta_index;  // built at the first zoom batch
    float bbox6[6] = {0, 0, 0, 0, 0, 0};  // xmin,xmax,ymin,ymax,zmin,zmax
    // octree + leaf deposit state
    Octree tree;
    bool has_tree = false;
    int leaf_dims = 16;
    std::vector<GridDesc> leaf_grids;
    std::vector<Item> leaf_items;
    std::vector<std::vector<int>> leaf_item_ranges;
    DevBuf<Item> d_items;
    DevBuf<GridDesc> d_grids;
    DevBuf<unsigned long long> d_fixed;
    DevBuf<double> d_out;
    DevBuf<int> d_counter;
    DevBuf<unsigned long long> d_stats;
    DevBuf<unsigned long long> d_route;  // ill-conditioned tets of a leaf deposit
    unsigned long long route_cap = 0;
    DevBuf<long long> d_cube_off;
    std::vector<long long> cube_off;
    size_t out_values = 0;
    cudaGraphExec_t graph_exec = nullptr;
    cudaGraph_t graph = nullptr;
    std::mutex mu;
    Tuning tuning;
    // zoom batches and the serving loop (serving.cuh), created at the first submit
    struct Server *server = nullptr;
    std::mutex server_mu;
};

static void server_destroy(adeco_session *s);

static void session_drop_graph(adeco_session *s)
{
    if (s->graph_exec) cudaGraphExecDestroy(s->graph_exec);
    if (s->graph) cudaGraphDestroy(s->graph);
    s->graph_exec = nullptr;
    s->graph = nullptr;
}

__global__ void xyz_to_float4_kernel(const float *xyz, float4 *out, long long n)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = make_float4(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], 0.f);
}

// Device, stream and kernel set-up of a new session (the lattice is filled by the caller).
static int session_open(const adeco_session_config *cfg, adeco_session &S)
{
    if (cfg) {
        S.device = cfg->device;
        S.order = cfg->tet_order;
        S.tet_mass = cfg->tet_mass > 0 ? cfg->tet_mass : 1.0;
        S.hbm_fraction = cfg->hbm_fraction > 0 ? cfg->hbm_fraction : 0.75;
        S.acc_fp64 = cfg->accumulate_fp64;
    }
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) return fail(ADECO_ERR_DEVICE, "no CUDA device");
    if (S.device < 0 || S.device >= count) return fail(ADECO_ERR_DEVICE, "invalid device %d", S.device);
    CUDA_TRY(cudaSetDevice(S.device));
    int rc = mixed_setup(S.device, S.dp);
    if (rc) return rc;
    CUDA_TRY(cudaStreamCreateWithFlags(&S.stream, cudaStreamNonBlocking));
    return ADECO_OK;
}

// Meta-cell AABBs of the resident lattice (MetaMesh), on the device; their
// union into bbox6 (xmin,xmax,...) when bbox6 is non-null.
static int session_meta_bbox(adeco_session &S, float *bbox6)
{
    S.meta.init(S.nx, S.ny, S.nz);
    const long long nmc = (long long)S.meta.count();
    DevBuf<float> &d_bb = S.d_meta_bbox;
    int rc;
    if ((rc = d_bb.reserve((size_t)nmc * 6))) return rc;
    meta_bbox_kernel<<<(unsigned)((nmc * 32 + 255) / 256), 256, 0, S.stream>>>(S.lattice.p, S.nx, S.ny, S.nz, S.meta.cd[0],
                                                                                  S.meta.cd[1], S.meta.cd[2], d_bb.p);
    CUDA_TRY(cudaGetLastError());
    S.meta.bbox.resize((size_t)nmc * 6);
    CUDA_TRY(cudaMemcpyAsync(S.meta.bbox.data(), d_bb.p, (size_t)nmc * 6 * sizeof(float), cudaMemcpyDeviceToHost,
                             S.stream));
    CUDA_TRY(cudaStreamSynchronize(S.stream));
    if (bbox6) {
        float mn[3] = {3.4e38f, 3.4e38f, 3.4e38f}, mx[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
        for (size_t i = 0; i < S.meta.count(); ++i)
            for (int a = 0; a < 3; ++a) {
                mn[a] = std::min(mn[a], S.meta.bbox[6 * i + a]);
                mx[a] = std::max(mx[a], S.meta.bbox[6 * i + 3 + a]);
            }
        for (int a = 0; a < 3; ++a) {
            bbox6[2 * a] = mn[a];
            bbox6[2 * a + 1] = mx[a];
        }
    }
    return ADECO_OK;
}

// Meta-cells, bounding box and work counters once the lattice is resident.
static int session_finish(adeco_session &S)
{
    int rc = session_meta_bbox(S, S.bbox6);
    if (rc) return rc;
    if ((rc = S.d_counter.reserve(2)) || (rc = S.d_stats.reserve(kNumStats))) return rc;
    CUDA_TRY(cudaMemset(S.d_counter.p, 0, 2 * sizeof(int)));
    return ADECO_OK;
}

#include "readers.cuh"
#include "octree_device.cuh"

// Reads `path` into the session's lattice (see readers.cuh).
static int read_particle_file(adeco_session &S, const char *path, int format, int stride, int periodic, float bbox_out[6])
{
    HostFile hf;
    hf.f = std::fopen(path, "rb");
    if (!hf.f) return fail(ADECO_ERR_ARGUMENT, "failed to open file: %s", path);
    std::fseek(hf.f, 0, SEEK_END);
    const long long fsize = (long long)std::ftell(hf.f);
    size_t first = 0, recsize = 12;
    long long count = 0;
    int n = 0, n0 = 0;
    if (format == ADECO_FORMAT_SORTED_BY_ID) {
        if (fsize % 12) return fail(ADECO_ERR_ARGUMENT, "inconsistent file size");
        count = fsize / 12;
        n0 = (int)std::llrint(std::cbrt((double)count));
        if ((long long)n0 * n0 * n0 != count) return fail(ADECO_ERR_ARGUMENT, "lagrangian grid not cubical");
        n = n0;  // the reference ignores the stride for this format
    } else if (format == ADECO_FORMAT_DARK_SKY) {
        int rc = sdf_header_size(hf.f, first);
        if (rc) return rc;
        recsize = 32;
        if ((long long)first > fsize || (fsize - (long long)first) % 32)
            return fail(ADECO_ERR_ARGUMENT, "inconsistent file size");
        count = (fsize - (long long)first) / 32;
        n0 = (int)std::llrint(std::cbrt((double)count));
        if ((long long)n0 * n0 * n0 != count) return fail(ADECO_ERR_ARGUMENT, "lagrangian grid not cubical");
        if (stride < 1 || n0 % stride) return fail(ADECO_ERR_ARGUMENT, "invalid stride %d for data dimensions %d", stride, n0);
        n = n0 / stride;
    } else {
        return fail(ADECO_ERR_ARGUMENT, "unknown particle file format %d", format);
    }
    if (n < 2) return fail(ADECO_ERR_ARGUMENT, "lattice must be at least 2^3 (got %d^3)", n);
    S.nx = S.ny = S.nz = n;
    const long long total = (long long)n * n * n;
    int rc;
    if ((rc = S.lattice.reserve((size_t)total))) return rc;
    DevBuf<unsigned long long> d_kept;
    DevBuf<int> d_err;
    if ((rc = d_kept.reserve(1)) || (rc = d_err.reserve(1))) return rc;
    CUDA_TRY(cudaMemsetAsync(d_kept.p, 0, sizeof(unsigned long long), S.stream));
    CUDA_TRY(cudaMemsetAsync(d_err.p, 0, sizeof(int), S.stream));
    ChunkPipe pipe;
    if ((rc = pipe.open())) return rc;
    const long long per_chunk = (long long)(kReadChunk / recsize);
    std::fseek(hf.f, (long)first, SEEK_SET);
    long long done = 0;
    for (int b = 0; done < count; b ^= 1) {
        const long long nrec = std::min(per_chunk, count - done);
        CUDA_TRY(cudaEventSynchronize(pipe.done[b]));  // this buffer's previous chunk is decoded
        if (std::fread(pipe.host[b], recsize, (size_t)nrec, hf.f) != (size_t)nrec)
            return fail(ADECO_ERR_ARGUMENT, "short read of %s", path);
        CUDA_TRY(cudaMemcpyAsync(pipe.dev[b], pipe.host[b], (size_t)nrec * recsize, cudaMemcpyHostToDevice, S.stream));
        const unsigned blocks = (unsigned)std::min<long long>((nrec + 255) / 256, 4096);
        if (format == ADECO_FORMAT_SORTED_BY_ID)
            sorted_chunk_kernel<<<blocks, 256, 0, S.stream>>>(reinterpret_cast<const float *>(pipe.dev[b]), done, nrec,
                                                              S.lattice.p);
        else
            darksky_chunk_kernel<<<blocks, 256, 0, S.stream>>>(pipe.dev[b], nrec, n0, stride, n, S.lattice.p, d_kept.p,
                                                               d_err.p);
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaEventRecord(pipe.done[b], S.stream));
        done += nrec;
    }
    CUDA_TRY(cudaStreamSynchronize(S.stream));
    if (format == ADECO_FORMAT_DARK_SKY) {
        unsigned long long kept = 0;
        int err = 0;
        CUDA_TRY(cudaMemcpy(&kept, d_kept.p, sizeof kept, cudaMemcpyDeviceToHost));
        CUDA_TRY(cudaMemcpy(&err, d_err.p, sizeof err, cudaMemcpyDeviceToHost));
        if (err) return fail(ADECO_ERR_ARGUMENT, "a particle id lies outside the %d^3 lattice", n0);
        if ((long long)kept != total)
            return fail(ADECO_ERR_ARGUMENT, "inconsistent global particle number (%llu of %lld)", kept, total);
    }
    // global bbox of the particles as read (the reference's global_bbox)
    float bb[6];
    if ((rc = session_meta_bbox(S, bb))) return rc;
    if (bbox_out)
        for (int k = 0; k < 6; ++k) bbox_out[k] = bb[k];
    if (periodic) {
        float e[3], lo[3], hi[3];
        for (int a = 0; a < 3; ++a) {
            const volatile float ext = bb[2 * a + 1] - bb[2 * a];  // FP32 steps, as the reference writes them
            const volatile float q = ext / 4.0f;
            const volatile float t = 0.75f * ext;
            e[a] = ext;
            lo[a] = bb[2 * a] + q;
            hi[a] = bb[2 * a] + t;
        }
        const float half = (float)n / 2.0f;
        unwrap_kernel<<<(unsigned)std::min<long long>((total + 255) / 256, 65535), 256, 0, S.stream>>>(
            S.lattice.p, n, half, make_float3(e[0], e[1], e[2]), make_float3(lo[0], lo[1], lo[2]),
            make_float3(hi[0], hi[1], hi[2]));
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaStreamSynchronize(S.stream));
    }
    return ADECO_OK;
}

extern "C" int adeco_session_create_from_file(const adeco_session_config *cfg, const char *path, int format, int stride,
                                              int periodic, float bbox_out[6], adeco_session **out)
{
    if (!out || !path) return fail(ADECO_ERR_ARGUMENT, "null path or output pointer");
    *out = nullptr;
    std::unique_ptr<adeco_session> s(new adeco_session());
    int rc = session_open(cfg, *s);
    if (rc) return rc;
    if ((rc = read_particle_file(*s, path, format, stride, periodic, bbox_out))) return rc;
    if ((rc = session_finish(*s))) return rc;
    *out = s.release();
    return ADECO_OK;
}

extern "C" int adeco_session_positions(adeco_session *s, float *xyz, size_t capacity)
{
    if (!s || !xyz) return fail(ADECO_ERR_ARGUMENT, "null argument");
    const size_t n = (size_t)s->nx * s->ny * s->nz;
    if (capacity < 3 * n) return fail(ADECO_ERR_ARGUMENT, "capacity %zu < %zu floats", capacity, 3 * n);
    CUDA_TRY(cudaSetDevice(s->device));
    std::vector<float4> tmp(n);
    CUDA_TRY(cudaMemcpy(tmp.data(), s->lattice.p, n * sizeof(float4), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n; ++i) {
        xyz[3 * i] = tmp[i].x;
        xyz[3 * i + 1] = tmp[i].y;
        xyz[3 * i + 2] = tmp[i].z;
    }
    return ADECO_OK;
}

extern "C" int adeco_session_lattice_dims(adeco_session *s, int dims[3])
{
    if (!s || !dims) return fail(ADECO_ERR_ARGUMENT, "null argument");
    dims[0] = s->nx;
    dims[1] = s->ny;
    dims[2] = s->nz;
    return ADECO_OK;
}

extern "C" int adeco_session_create(const adeco_session_config *cfg, const float *positions, int nx, int ny, int nz,
                                    adeco_session **out)
{
    if (!out || !positions) return fail(ADECO_ERR_ARGUMENT, "null positions or output pointer");
    *out = nullptr;
    if (nx < 2 || ny < 2 || nz < 2) return fail(ADECO_ERR_ARGUMENT, "lattice must be at least 2^3 (got %d,%d,%d)", nx, ny, nz);
    std::unique_ptr<adeco_session> s(new adeco_session());
    int rc = session_open(cfg, *s);
    if (rc) return rc;
    s->nx = nx; s->ny = ny; s->nz = nz;
    const long long n = (long long)nx * ny * nz;
    if ((rc = s->lattice.reserve((size_t)n))) return rc;
    {
        // Page-locked host positions are read by the conversion kernel itself
        // (one pass over the host link, no staging buffer); pageable ones are
        // copied to a device staging buffer first.
        cudaPointerAttributes at{};
        const float *src = nullptr;
        if (cudaPointerGetAttributes(&at, positions) == cudaSuccess && at.type == cudaMemoryTypeHost && at.devicePointer)
            src = static_cast<const float *>(at.devicePointer);
        else
            cudaGetLastError();  // clear the query's error for an unregistered pointer
        DevBuf<float> raw;
        if (!src) {
            if ((rc = raw.reserve((size_t)n * 3))) return rc;
            CUDA_TRY(cudaMemcpyAsync(raw.p, positions, (size_t)n * 3 * sizeof(float), cudaMemcpyHostToDevice, s->stream));
            src = raw.p;
        }
        xyz_to_float4_kernel<<<std::min<long long>((n + 255) / 256, 65535), 256, 0, s->stream>>>(src, s->lattice.p, n);
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaStreamSynchronize(s->stream));
    }
    if ((rc = session_finish(*s))) return rc;
    *out = s.release();
    return ADECO_OK;
}

extern "C" int adeco_session_destroy(adeco_session *s)
{
    if (!s) return ADECO_OK;
    cudaSetDevice(s->device);
    server_destroy(s);
    if (s->stream) cudaStreamSynchronize(s->stream);
    session_drop_graph(s);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return ADECO_OK;
}

extern "C" int adeco_session_bbox(adeco_session *s, float bbox[6])
{
    if (!s || !bbox) return fail(ADECO_ERR_ARGUMENT, "null argument");
    std::memcpy(bbox, s->bbox6, sizeof(s->bbox6));
    return ADECO_OK;
}

extern "C" int adeco_session_build_octree(adeco_session *s, const float *box6, const float *roi6,
                                          uint64_t max_tets_per_node, int max_level, int leaf_dims)
{
    if (!s) return fail(ADECO_ERR_ARGUMENT, "null session");
    if (leaf_dims < 1 || leaf_dims > 256) return fail(ADECO_ERR_ARGUMENT, "leaf_dims %d out of [1,256]", leaf_dims);
    if (max_level < 0) return fail(ADECO_ERR_ARGUMENT, "max_level must be >= 0");
    float box[6];
    if (box6) {
        std::memcpy(box, box6, sizeof box);
    } else {
        for (int a = 0; a < 3; ++a) {
            box[a] = s->bbox6[2 * a];
            box[3 + a] = s->bbox6[2 * a + 1];
        }
    }
    std::lock_guard<std::mutex> lk(s->mu);
    session_drop_graph(s);
    s->has_tree = false;
    // max_tets_per_node = min(global tets / ranks, parameter) (src/AdDepositWorkFlow.h:169), one rank
    const uint64_t total_tets = 6ull * (uint64_t)(s->nx - 1) * (uint64_t)(s->ny - 1) * (uint64_t)(s->nz - 1);
    const uint64_t max_tets = std::min(total_tets, max_tets_per_node);
    if (s->octree_builder == ADECO_OCTREE_DEVICE) {
        CUDA_TRY(cudaSetDevice(s->device));
        const int rc = build_octree_device(s->meta, s->d_meta_bbox.p, box, roi6, max_tets, max_level, s->stream, s->tree);
        if (rc) return rc;
    } else if (!s->tree.build(s->meta, box, roi6, max_tets, max_level)) {
        return fail(ADECO_ERR_LIMIT, "octree generation did not terminate");
    }
    s->leaf_dims = leaf_dims;
    // per-leaf grids and work items (leaf x meta-cell)
    const size_t nl = s->tree.leaves.size();
    const long long cells = (long long)leaf_dims * leaf_dims * leaf_dims;
    s->leaf_grids.resize(nl);
    const size_t n_items = (size_t)s->tree.leaf_meta_off[nl];
    s->leaf_items.resize(n_items);
    s->cube_off.resize(n_items + 1);
    long long cubes = 0;
    for (size_t q = 0; q < nl; ++q) {
        const OctNode &nd = s->tree.nodes[s->tree.leaves[q]];
        const float bb[6] = {nd.min[0], nd.min[0] + nd.ext, nd.min[1], nd.min[1] + nd.ext, nd.min[2], nd.min[2] + nd.ext};
        const int64_t m0 = s->tree.leaf_meta_off[q], m1 = s->tree.leaf_meta_off[q + 1];
        const int shift = choose_shift(2058.0 * (double)std::max<int64_t>(1, m1 - m0), s->tet_mass);
        s->leaf_grids[q] = make_grid(bb, leaf_dims, s->tet_mass, shift, (long long)q * cells);
        for (int64_t k = m0; k < m1; ++k) {
            int org[3], nv[3];
            s->meta.range(s->tree.leaf_meta_ids[k], org, nv);
            Item &it = s->leaf_items[k];
            it.base = org[0] + (long long)s->nx * (org[1] + (long long)s->ny * org[2]);
            it.grid = (int)q;
            it.nv = nv[0] | (nv[1] << 8) | (nv[2] << 16);
            s->cube_off[k] = cubes;
            cubes += (long long)(nv[0] - 1) * (nv[1] - 1) * (nv[2] - 1);
        }
    }
    s->cube_off[n_items] = cubes;
    int rc;
    s->out_values = nl * (size_t)cells;
    s->route_cap = route_capacity((long long)s->leaf_items.size());
    if ((rc = s->d_items.reserve(s->leaf_items.size())) || (rc = s->d_grids.reserve(nl)) ||
        (rc = s->d_fixed.reserve(s->out_values)) || (rc = s->d_out.reserve(s->out_values)) ||
        (rc = s->d_cube_off.reserve(s->cube_off.size())) || (rc = s->d_route.reserve(s->route_cap + 1)))
        return rc;
    CUDA_TRY(cudaMemcpyAsync(s->d_items.p, s->leaf_items.data(), s->leaf_items.size() * sizeof(Item),
                             cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(cudaMemcpyAsync(s->d_grids.p, s->leaf_grids.data(), nl * sizeof(GridDesc), cudaMemcpyHostToDevice,
                             s->stream));
    CUDA_TRY(cudaMemcpyAsync(s->d_cube_off.p, s->cube_off.data(), s->cube_off.size() * sizeof(long long),
                             cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    s->has_tree = true;
    return ADECO_OK;
}

extern "C" int adeco_session_set_octree_builder(adeco_session *s, int builder)
{
    if (!s) return fail(ADECO_ERR_ARGUMENT, "null session");
    if (builder != ADECO_OCTREE_DEVICE && builder != ADECO_OCTREE_HOST)
        return fail(ADECO_ERR_ARGUMENT, "unknown octree builder %d", builder);
    std::lock_guard<std::mutex> lk(s->mu);
    s->octree_builder = builder;
    return ADECO_OK;
}

extern "C" int adeco_session_octree_size(adeco_session *s, int *n_nodes, int *n_leaves, int *n_levels)
{
    if (!s) return fail(ADECO_ERR_ARGUMENT, "null session");
    if (!s->has_tree) return fail(ADECO_ERR_STATE, "no octree built");
    if (n_nodes) *n_nodes = (int)s->tree.nodes.size();
    if (n_leaves) *n_leaves = (int)s->tree.leaves.size();
    if (n_levels) *n_levels = s->tree.levels;
    return ADECO_OK;
}

extern "C" int adeco_session_octree_nodes(adeco_session *s, adeco_node *nodes, int capacity)
{
    if (!s || !nodes) return fail(ADECO_ERR_ARGUMENT, "null argument");
    if (!s->has_tree) return fail(ADECO_ERR_STATE, "no octree built");
    if (capacity < (int)s->tree.nodes.size()) return fail(ADECO_ERR_ARGUMENT, "capacity too small");
    std::vector<int> nmeta(s->tree.nodes.size(), 0);
    for (size_t q = 0; q < s->tree.leaves.size(); ++q)
        nmeta[s->tree.leaves[q]] = (int)(s->tree.leaf_meta_off[q + 1] - s->tree.leaf_meta_off[q]);
    for (size_t i = 0; i < s->tree.nodes.size(); ++i) {
        const OctNode &n = s->tree.nodes[i];
        adeco_node &o = nodes[i];
        o.min[0] = n.min[0]; o.min[1] = n.min[1]; o.min[2] = n.min[2];
        o.ext = n.ext;
        o.level = n.level;
        o.parent = n.parent;
        o.first_child = n.first_child;
        o.n_meta = nmeta[i];
        o.estimate = n.estimate;
    }
    return ADECO_OK;
}

extern "C" int adeco_session_leaves(adeco_session *s, int32_t *leaf_ids, int capacity)
{
    if (!s || !leaf_ids) return fail(ADECO_ERR_ARGUMENT, "null argument");
    if (!s->has_tree) return fail(ADECO_ERR_STATE, "no octree built");
    if (capacity < (int)s->tree.leaves.size()) return fail(ADECO_ERR_ARGUMENT, "capacity too small");
    std::copy(s->tree.leaves.begin(), s->tree.leaves.end(), leaf_ids);
    return ADECO_OK;
}

extern "C" int adeco_session_leaf_meta(adeco_session *s, int leaf_index, uint64_t *ids, int capacity, int *count)
{
    if (!s || !count) return fail(ADECO_ERR_ARGUMENT, "null argument");
    if (!s->has_tree) return fail(ADECO_ERR_STATE, "no octree built");
    if (leaf_index < 0 || leaf_index >= (int)s->tree.leaves.size()) return fail(ADECO_ERR_ARGUMENT, "bad leaf index");
    const int64_t a = s->tree.leaf_meta_off[leaf_index], b = s->tree.leaf_meta_off[leaf_index + 1];
    *count = (int)(b - a);
    if (ids) {
        if (capacity < *count) return fail(ADECO_ERR_ARGUMENT, "capacity too small");
        std::copy(s->tree.leaf_meta_ids.begin() + a, s->tree.leaf_meta_ids.begin() + b, ids);
    }
    return ADECO_OK;
}

static DepositParams session_params(adeco_session *s, bool stats)
{
    DepositParams P = base_params(s->tuning);
    P.items = s->d_items.p;
    P.n_items = (int)s->leaf_items.size();
    P.src_kind = SRC_LATTICE_F4;
    P.grids = s->d_grids.p;
    P.src = s->lattice.p;
    P.stride_y = s->nx;
    P.stride_z = (long long)s->nx * s->ny;
    P.order = s->order;
    P.pad_check = 0;
    P.out = s->d_fixed.p;
    P.out_d = s->d_out.p;
    P.counter = s->d_counter.p;
    P.error = s->d_counter.p + 1;
    P.stats = stats ? s->d_stats.p : nullptr;
    set_route(P, s->d_route.p, s->tuning.route_capacity ? std::min(s->tuning.route_capacity, s->route_cap)
                                                          : s->route_cap);
    return P;
}

// enqueue the batched leaf deposit (memset, persistent kernel, conversion)
static int enqueue_leaves_mixed(adeco_session *s, bool stats)
{
    const size_t nv = s->out_values;
    CUDA_TRY(cudaMemsetAsync(s->d_fixed.p, 0, nv * sizeof(unsigned long long), s->stream));
    int rc = launch_mixed(s->dp, session_params(s, stats), false, s->stream, s->tuning.ctas_per_sm);
    if (rc) return rc;
    const long long cells = (long long)s->leaf_dims * s->leaf_dims * s->leaf_dims;
    fixed_to_f64_grids_kernel<<<s->dp.sms * 4, 256, 0, s->stream>>>(s->d_fixed.p, s->d_out.p, s->d_grids.p,
                                                                    (int)s->leaf_grids.size(), cells);
    CUDA_TRY(cudaGetLastError());
    return ADECO_OK;
}

extern "C" int adeco_session_deposit_leaves(adeco_session *s, int precision, double *host_out, int collect_stats,
                                            adeco_timing *timing)
{
    if (!s) return fail(ADECO_ERR_ARGUMENT, "null session");
    if (!s->has_tree) return fail(ADECO_ERR_STATE, "no octree built");
    std::lock_guard<std::mutex> lk(s->mu);
    CUDA_TRY(cudaSetDevice(s->device));
    cudaEvent_t e0, e1, e2;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    CUDA_TRY(cudaEventCreate(&e2));
    if (collect_stats) CUDA_TRY(cudaMemsetAsync(s->d_stats.p, 0, kNumStats * sizeof(unsigned long long), s->stream));
    uint64_t launches = 0;
    int rc = ADECO_OK;
    if (precision == ADECO_PREC_FP64) {
        const size_t nv = s->out_values;
        CUDA_TRY(cudaMemsetAsync(s->d_out.p, 0, nv * sizeof(double), s->stream));
        CUDA_TRY(cudaEventRecord(e0, s->stream));
        // one launch per leaf (one request per launch)
        DepositParams P = session_params(s, false);
        size_t item0 = 0;
        for (size_t q = 0; q < s->leaf_grids.size() && !rc; ++q) {
            size_t item1 = item0;
            while (item1 < s->leaf_items.size() && s->leaf_items[item1].grid == (int)q) ++item1;
            DepositParams Q = P;
            Q.items = s->d_items.p + item0;
            Q.n_items = (int)(item1 - item0);
            const long long c0 = s->cube_off[item0], c1 = s->cube_off[item1];
            if (Q.n_items > 0 && c1 > c0) {
                rc = launch_plain(s->dp, Q, s->d_cube_off.p + item0, c0, c1, s->stream);
                ++launches;
            }
            item0 = item1;
        }
        CUDA_TRY(cudaEventRecord(e1, s->stream));
        CUDA_TRY(cudaEventRecord(e2, s->stream));
    } else {
        CUDA_TRY(cudaMemsetAsync(s->d_fixed.p, 0, s->out_values * sizeof(unsigned long long), s->stream));
        CUDA_TRY(cudaEventRecord(e0, s->stream));
        rc = launch_mixed(s->dp, session_params(s, collect_stats != 0), false, s->stream, s->tuning.ctas_per_sm);
        launches = 2;  // the mixed kernel and the ill-conditioned-tet launch
        CUDA_TRY(cudaEventRecord(e1, s->stream));
        const long long cells = (long long)s->leaf_dims * s->leaf_dims * s->leaf_dims;
        fixed_to_f64_grids_kernel<<<s->dp.sms * 4, 256, 0, s->stream>>>(s->d_fixed.p, s->d_out.p, s->d_grids.p,
                                                                        (int)s->leaf_grids.size(), cells);
        ++launches;
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaEventRecord(e2, s->stream));
    }
    if (rc) return rc;
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    int err = 0;
    CUDA_TRY(cudaMemcpy(&err, s->d_counter.p + 1, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) {
        cudaMemset(s->d_counter.p + 1, 0, sizeof(int));
        return deposit_error(err, "a leaf grid");
    }
    unsigned long long routed = 0;  // the mixed launch's route list count
    if (precision != ADECO_PREC_FP64)
        CUDA_TRY(cudaMemcpy(&routed, s->d_route.p, sizeof routed, cudaMemcpyDeviceToHost));
    float k_ms = 0.f, t_ms = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&k_ms, e0, e1));
    CUDA_TRY(cudaEventElapsedTime(&t_ms, e0, e2));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(e2);
    if (timing) {
        std::memset(timing, 0, sizeof *timing);
        timing->kernel_ms = k_ms;
        timing->total_ms = t_ms;
        timing->launches = launches;
        timing->items = s->leaf_items.size();
        timing->routed_tets = routed;
        if (collect_stats) {
            unsigned long long st[kNumStats];
            CUDA_TRY(cudaMemcpy(st, s->d_stats.p, sizeof st, cudaMemcpyDeviceToHost));
            timing->tets = st[ST_TETS];
            timing->candidate_pairs = st[ST_CAND];
            timing->partial_pairs = st[ST_PARTIAL];
            timing->cell_inside_pairs = st[ST_CELLIN];
            timing->tet_inside_pairs = st[ST_INSIDE];
            timing->fp64_pairs = st[ST_FP64];
            timing->serial_pieces = st[ST_FALLBACK];
        }
    }
    if (host_out) CUDA_TRY(cudaMemcpy(host_out, s->d_out.p, s->out_values * sizeof(double), cudaMemcpyDeviceToHost));
    return ADECO_OK;
}

extern "C" int adeco_session_leaf_grids_device(adeco_session *s, const double **d_grids, size_t *n_values)
{
    if (!s || !d_grids || !n_values) return fail(ADECO_ERR_ARGUMENT, "null argument");
    if (!s->has_tree) return fail(ADECO_ERR_STATE, "no octree built");
    *d_grids = s->d_out.p;
    *n_values = s->out_values;
    return ADECO_OK;
}

extern "C" int adeco_session_replay_leaves(adeco_session *s, int reps, adeco_timing *timing)
{
    if (!s) return fail(ADECO_ERR_ARGUMENT, "null session");
    if (!s->has_tree) return fail(ADECO_ERR_STATE, "no octree built");
    if (reps < 1) return fail(ADECO_ERR_ARGUMENT, "reps must be >= 1");
    std::lock_guard<std::mutex> lk(s->mu);
    CUDA_TRY(cudaSetDevice(s->device));
    if (!s->graph_exec) {
        CUDA_TRY(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
        int rc = enqueue_leaves_mixed(s, false);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(s->stream, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return fail(ADECO_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
        s->graph = g;
        CUDA_TRY(cudaGraphInstantiate(&s->graph_exec, s->graph, 0));
    }
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    CUDA_TRY(cudaEventRecord(e0, s->stream));
    for (int r = 0; r < reps; ++r) CUDA_TRY(cudaGraphLaunch(s->graph_exec, s->stream));
    CUDA_TRY(cudaEventRecord(e1, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    float ms = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (timing) {
        std::memset(timing, 0, sizeof *timing);
        timing->kernel_ms = ms / reps;
        timing->total_ms = ms / reps;
        timing->launches = 3ull * reps;
        timing->items = s->leaf_items.size();
    }
    return ADECO_OK;
}

// ============================================================ diagnostics
extern "C" int adeco_debug_tet_records(const float *positions, size_t positions_size, int m, size_t cube_begin,
                                       size_t cube_end, const float bbox[6], int dims, int tet_order, int32_t *records,
                                       uint32_t *cand)
{
    if (!positions || !bbox || m < 1 || dims < 1) return fail(ADECO_ERR_ARGUMENT, "bad arguments");
    const size_t fpp = 3 * (size_t)(m + 1) * (m + 1) * (m + 1);
    if (positions_size % fpp) return fail(ADECO_ERR_ARGUMENT, "positions_size not a multiple of the patch size");
    const size_t cubes_total = positions_size / fpp * (size_t)m * m * m;
    if (cube_end > cubes_total || cube_begin > cube_end) return fail(ADECO_ERR_ARGUMENT, "cube range out of bounds");
    int dev = 0;
    int rc = select_device(0, 0, dev);
    if (rc) return rc;
    const size_t ncube = cube_end - cube_begin;
    const size_t ncell = (size_t)dims * dims * dims;
    DevBuf<float> d_pos;
    DevBuf<int> d_rec;
    DevBuf<unsigned int> d_cand;
    if ((rc = d_pos.reserve(positions_size)) || (rc = d_rec.reserve(std::max<size_t>(1, ncube * 6 * 13))) ||
        (rc = d_cand.reserve(ncell)))
        return rc;
    CUDA_TRY(cudaMemcpy(d_pos.p, positions, positions_size * sizeof(float), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemset(d_cand.p, 0, ncell * sizeof(unsigned int)));
    const GridDesc g = make_grid(bbox, dims, 1.0, 32, 0);
    if (ncube) {
        tet_records_kernel<<<(unsigned)((ncube + 127) / 128), 128>>>(d_pos.p, m, (long long)cube_begin,
                                                                     (long long)cube_end, g, tet_order, d_rec.p,
                                                                     cand ? d_cand.p : nullptr);
        CUDA_TRY(cudaGetLastError());
    }
    CUDA_TRY(cudaDeviceSynchronize());
    if (records && ncube) CUDA_TRY(cudaMemcpy(records, d_rec.p, ncube * 6 * 13 * sizeof(int), cudaMemcpyDeviceToHost));
    if (cand) CUDA_TRY(cudaMemcpy(cand, d_cand.p, ncell * sizeof(unsigned int), cudaMemcpyDeviceToHost));
    return ADECO_OK;
}

// ============================================================ zoom batches and serving
#include "serving.cuh"

// ============================================================ bounded waits
// One warp waits, through wait_zero_bounded (the wait every spin of the
// deposit kernels uses), on a count that nothing decrements; when the limit
// runs out it sets error bit 3, as the work-sharing wait does, and returns.
__global__ void bounded_wait_kernel(int *error, unsigned spins)
{
    __shared__ int busy;
    if (threadIdx.x == 0) busy = 1;
    __syncwarp();
    if (threadIdx.x == 0 && !wait_zero_bounded(&busy, spins, 32)) atomicOr(error, 8);
}

extern "C" int adeco_debug_bounded_wait(unsigned spins)
{
    if (spins > (1u << 26)) return fail(ADECO_ERR_ARGUMENT, "spins %u above 2^26", spins);
    int dev = 0;
    int rc = select_device(0, 0, dev);
    if (rc) return rc;
    DevBuf<int> d_err;
    if ((rc = d_err.reserve(1))) return rc;
    CUDA_TRY(cudaMemset(d_err.p, 0, sizeof(int)));
    bounded_wait_kernel<<<1, 32>>>(d_err.p, spins);
    CUDA_TRY(cudaGetLastError());
    int err = 0;
    CUDA_TRY(cudaMemcpy(&err, d_err.p, sizeof err, cudaMemcpyDeviceToHost));
    if (err) return deposit_error(err, "the bounded-wait check");
    return ADECO_OK;
}

// ============================================================ peak probe
// FP32 FMA throughput of this device: 8 independent FMA chains per thread,
// enough warps to fill every SM; reported as TFLOP/s (2 flops per FMA).
__global__ void fma_probe_kernel(float *out, int iters, float a, float b)
{
    float x0 = threadIdx.x * 1e-3f, x1 = x0 + 1.f, x2 = x0 + 2.f, x3 = x0 + 3.f;
    float x4 = x0 + 4.f, x5 = x0 + 5.f, x6 = x0 + 6.f, x7 = x0 + 7.f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
            x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
        }
    }
    const float r = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (r == 12345.678f) out[blockIdx.x] = r;  // keeps the chains alive
}

extern "C" int adeco_probe_fp32_tflops(int device, double *tflops)
{
    if (!tflops) return fail(ADECO_ERR_ARGUMENT, "null output");
    CUDA_TRY(cudaSetDevice(device));
    cudaDeviceProp prop;
    CUDA_TRY(cudaGetDeviceProperties(&prop, device));
    DevBuf<float> out;
    int rc = out.reserve(4096);
    if (rc) return rc;
    const int blocks = prop.multiProcessorCount * 8, threads = 256, iters = 2048;
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    double best = 0.0;
    for (int rep = 0; rep < 5; ++rep) {
        CUDA_TRY(cudaEventRecord(e0));
        fma_probe_kernel<<<blocks, threads>>>(out.p, iters, 0.999f, 1e-4f);
        CUDA_TRY(cudaEventRecord(e1));
        CUDA_TRY(cudaEventSynchronize(e1));
        float ms = 0.f;
        CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
        const double flops = 2.0 * 8 * 16 * (double)iters * blocks * threads;
        if (rep > 0) best = std::max(best, flops / (ms * 1e-3) / 1e12);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *tflops = best;
    return ADECO_OK;
}

// ============================================================ no-allocation entry point
// adeco_deposit_tets_device_noalloc: the mixed deposit of
// adeco_deposit_tets_device for callers that must not allocate device memory
// while they deposit -- an application that hands all of the GPU's memory to
// its own pool at start-up, or a latency-critical loop in which cudaMalloc's
// unbounded time and cudaFree's device-wide synchronisation are not allowed.
// Its scratch -- work counter, error flag, grid descriptor, work items, the
// 64-bit fixed-point accumulators and the list of ill-conditioned tets --
// lives in one file-scope device array of kNoAllocScratchBytes (15.5 MB)
// that every GPU loading this library holds until the process exits.  The
// array is shared by every call on a device and keeps the last call's
// contents; each call clears what must start at zero.  Calls that overlap on
// the GPU (two streams, or two host threads) race on it: serialise them.
namespace {
constexpr int kNoAllocMaxItems = 4096;                  // patch sub-blocks of <= 7^3 cubes
constexpr long long kNoAllocMaxCells = 96LL * 96 * 96;  // grid cells (dims <= 96 for a cube)
constexpr size_t kNoAllocHeader = 1024;                 // counter, error flag, GridDesc
// ill-conditioned tets per call: the allocating path's rule at the item limit,
// so both paths accept the same calls
constexpr unsigned long long kNoAllocRouteCap = route_capacity(kNoAllocMaxItems);
constexpr size_t kNoAllocScratchBytes = kNoAllocHeader + (size_t)kNoAllocMaxItems * sizeof(Item) +
                                        (size_t)kNoAllocMaxCells * sizeof(unsigned long long) +
                                        (size_t)(kNoAllocRouteCap + 1) * sizeof(unsigned long long);
}  // namespace

static_assert(kNoAllocRouteCap == 1048576ull, "route list of the no-alloc scratch: 2^20 entries");
static_assert(256 + sizeof(GridDesc) <= kNoAllocHeader, "grid descriptor must fit the scratch header");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {
struct NoAllocDevice {
    bool ready = false;
    unsigned char *scratch = nullptr;  // device address of g_noalloc_scratch
    int sms = 0;
    int blocks_per_sm = 0;
};
constexpr int kNoAllocMaxDevices = 64;
NoAllocDevice g_noalloc_dev[kNoAllocMaxDevices];
std::mutex g_noalloc_mu;

// once per device, with that device current
int noalloc_setup(int dev, NoAllocDevice &out)
{
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    NoAllocDevice &d = g_noalloc_dev[dev];
    if (!d.ready) {
        void *ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || ptr == nullptr)
            return fail(ADECO_ERR_CUDA, "cudaGetSymbolAddress of the no-alloc scratch failed: %s",
                        cudaGetErrorString(e));
        int sms = 0, nb = 0;
        CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        CUDA_TRY(cudaFuncSetAttribute(deposit_mixed_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)sizeof(SharedMixed)));
        CUDA_TRY(cudaFuncSetAttribute(route_fp64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRouteSmem));
        CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, deposit_mixed_kernel<false>, kThreads,
                                                               sizeof(SharedMixed)));
        d.scratch = static_cast<unsigned char *>(ptr);
        d.sms = sms;
        d.blocks_per_sm = nb > 0 ? nb : 1;
        d.ready = true;
    }
    out = d;
    return ADECO_OK;
}
}  // namespace

// the grid descriptor, passed by value, into the scratch
__global__ void noalloc_grid_kernel(GridDesc *dst, GridDesc g) { *dst = g; }

// work items of patches [p0, p0 + np): sub-blocks of <= 7^3 cubes, as patch_items()
__global__ void noalloc_items_kernel(Item *items, long long p0, int n_items, int m, int nsb)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_items) return;
    const long long n1 = m + 1, n2 = n1 * n1;
    const int per = nsb * nsb * nsb;
    const long long p = p0 + i / per;
    const int sb = i % per, sx = sb % nsb, sy = (sb / nsb) % nsb, sz = sb / (nsb * nsb);
    const int ox = sx * kMetaCubes, oy = sy * kMetaCubes, oz = sz * kMetaCubes;
    const int vx = min(kMetaCubes + 1, m + 1 - ox), vy = min(kMetaCubes + 1, m + 1 - oy),
              vz = min(kMetaCubes + 1, m + 1 - oz);
    Item it;
    it.base = p * n1 * n2 + ox + n1 * oy + n2 * oz;
    it.grid = 0;
    it.nv = vx | (vy << 8) | (vz << 16);
    items[i] = it;
}

extern "C" int adeco_deposit_tets_device_noalloc(const float *d_positions, size_t positions_size, size_t patch_offset,
                                                 size_t num_patches, int meta_cells_per_patch, const float bbox[6],
                                                 int dims, double *d_out, int tet_order, double tet_mass, void *stream)
{
    if (positions_size == 0 || num_patches == 0) return ADECO_OK;
    const int m = meta_cells_per_patch;
    int rc = validate_boundary(patch_offset, num_patches, d_positions, positions_size, m, bbox, dims, d_out);
    if (rc) return rc;
    if (tet_order != ADECO_ORDER_REF && tet_order != ADECO_ORDER_CONFORMING)
        return fail(ADECO_ERR_ARGUMENT, "unknown tet order %d", tet_order);
    const long long ncell = (long long)dims * dims * dims;
    if (ncell > kNoAllocMaxCells)
        return fail(ADECO_ERR_LIMIT, "no-alloc deposit: %lld grid cells exceed the fixed scratch of %lld cells "
                    "(dims <= 96)", ncell, kNoAllocMaxCells);
    const int nsb = MetaGrid::ceil_div(m, kMetaCubes);
    const long long n_items = (long long)num_patches * nsb * nsb * nsb;
    if (n_items > kNoAllocMaxItems)
        return fail(ADECO_ERR_LIMIT, "no-alloc deposit: %lld work items exceed the fixed scratch of %d "
                    "(patches x ceil(m/7)^3)", n_items, kNoAllocMaxItems);
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(ADECO_ERR_DEVICE, "device %d out of range", dev);
    NoAllocDevice nd;
    if ((rc = noalloc_setup(dev, nd))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    int *counter = reinterpret_cast<int *>(nd.scratch);  // [0] work counter, [1] error flag
    GridDesc *grid = reinterpret_cast<GridDesc *>(nd.scratch + 256);
    Item *items = reinterpret_cast<Item *>(nd.scratch + kNoAllocHeader);
    unsigned long long *fixed =
        reinterpret_cast<unsigned long long *>(nd.scratch + kNoAllocHeader + (size_t)kNoAllocMaxItems * sizeof(Item));
    unsigned long long *route = fixed + kNoAllocMaxCells;  // count word, then the entries
    const int shift = choose_shift(6.0 * (double)num_patches * (double)m * m * m, tet_mass);
    CUDA_TRY(cudaMemsetAsync(counter, 0, 2 * sizeof(int), st));
    CUDA_TRY(cudaMemsetAsync(route, 0, sizeof(unsigned long long), st));
    CUDA_TRY(cudaMemsetAsync(fixed, 0, (size_t)ncell * sizeof(unsigned long long), st));
    noalloc_grid_kernel<<<1, 1, 0, st>>>(grid, make_grid(bbox, dims, tet_mass, shift, 0));
    noalloc_items_kernel<<<(unsigned)((n_items + 127) / 128), 128, 0, st>>>(items, (long long)patch_offset,
                                                                           (int)n_items, m, nsb);
    CUDA_TRY(cudaGetLastError());
    DepositParams P = base_params(Tuning());
    P.items = items;
    P.n_items = (int)n_items;
    P.src_kind = SRC_PATCH_F3;
    P.grids = grid;
    P.src = d_positions;
    P.stride_y = m + 1;
    P.stride_z = (long long)(m + 1) * (m + 1);
    P.order = tet_order;
    P.pad_check = 1;
    P.out = fixed;
    P.counter = counter;
    P.error = counter + 1;
    set_route(P, route, route_capacity(n_items));  // <= kNoAllocRouteCap, the allocating path's rule
    const int blocks = (int)std::max(1LL, std::min(n_items, (long long)nd.sms * nd.blocks_per_sm));
    deposit_mixed_kernel<false><<<blocks, kThreads, sizeof(SharedMixed), st>>>(P);
    CUDA_TRY(cudaGetLastError());
    route_fp64_kernel<<<nd.sms * 2, kThreads, kRouteSmem, st>>>(P);  // the resident CTAs
    CUDA_TRY(cudaGetLastError());
    fixed_accumulate_f64_kernel<<<1024, 256, 0, st>>>(fixed, d_out, ncell, std::ldexp(1.0, -shift));
    CUDA_TRY(cudaGetLastError());
    int err = 0;
    CUDA_TRY(cudaMemcpyAsync(&err, counter + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (err) return deposit_error(err, "the grid");
    return ADECO_OK;
}
