/*
 * adeco_deposit.h -- C ABI of the GB300-native phase-space tetrahedron mass
 * deposit (libadeco_gb300.so).
 *
 * Plain C types only (pointers, sizes, PODs): any host language binds it
 * through its FFI.  Every entry point returns an adeco_status_code and never
 * exits the process; adeco_last_error() gives the message of the calling
 * thread's last failure.
 *
 * Reference interfaces replaced (paths within kaehlerr/ADECO):
 *   adeco_deposit_tets     <- AdaptiveMassDeposit::DepositWrapper::deposit_tets
 *                             src/AdDeposit2Grid.h:82-91 (CPU src/AdDeposit2Grid.cpp:67,
 *                             GPU src/AdDeposit2Grid.cu:543 -> resample() :229)
 *   adeco_deposit_tets_ex  <- the same boundary, with FP64 output and the
 *                             precision / tet-order / mass options
 *   adeco_session_*        <- the state deposit_workflow keeps across its phases
 *                             (src/AdDepositWorkFlow.h:60-237): the particle
 *                             lattice (Tetrahedra, MetaMesh) and the octree
 *   adeco_session_build_octree
 *                          <- AdOctreeGeneration::generate_tree
 *                             src/AdOctreeGeneration.h:76-208 with
 *                             MetaMesh::get_estimate_num_tets src/AdTypeDefinitions.h:812
 *   adeco_session_deposit_leaves
 *                          <- deposit_leaf_nodes src/AdDynamicLoadBalancing.h:983-1323
 *                             (single rank), without the file writer
 *   adeco_session_submit / _poll / _wait / _result
 *                          <- no counterpart: batched zoom requests and the
 *                             serving loop (continuous batching)
 */
#ifndef ADECO_DEPOSIT_H
#define ADECO_DEPOSIT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ADECO_ABI_VERSION 2

typedef enum {
    ADECO_OK = 0,
    ADECO_ERR_ARGUMENT = 1,   /* invalid argument (null pointer, bad size, ...)          */
    ADECO_ERR_OVERFLOW = 2,   /* counts overflow the reference's int cube counter        */
    ADECO_ERR_DEVICE = 3,     /* no CUDA device / invalid device id                      */
    ADECO_ERR_CUDA = 4,       /* a CUDA runtime call failed                              */
    ADECO_ERR_MEMORY = 5,     /* not enough device memory (admission refused)            */
    ADECO_ERR_INCONSISTENT = 6, /* patch_offset + num_patches beyond the positions array */
    ADECO_ERR_STATE = 7,      /* call out of order (e.g. no octree built yet)            */
    ADECO_ERR_NOT_FOUND = 8,  /* unknown batch / request id                              */
    ADECO_ERR_LIMIT = 9       /* a documented size limit was exceeded                    */
} adeco_status_code;

typedef enum { ADECO_PREC_MIXED = 0, ADECO_PREC_FP64 = 1 } adeco_precision;
typedef enum { ADECO_ORDER_REF = 0, ADECO_ORDER_CONFORMING = 1 } adeco_tet_order;
typedef enum { ADECO_OUT_F32 = 0, ADECO_OUT_F64 = 1 } adeco_out_type;

/* Thread-local message of the last failed call ("" if none). */
const char *adeco_last_error(void);
int adeco_abi_version(void);

/* ------------------------------------------------------------------ */
/* The reference boundary                                              */
/*
 * Deposit the tets of patches [patch_offset, patch_offset+num_patches) of
 * `positions` (host memory; each patch is (m+1)^3 vertices x 3 floats, x
 * fastest, 666.f marks padding vertices) into the dims^3 grid over bbox
 * (xmin,xmax,ymin,ymax,zmin,zmax), ACCUMULATING (+=) into `data` (host,
 * float, x fastest).  Mass 1 per tet, the reference's tet construction.
 * `use_specific_gpu` / `device_id` select the CUDA device as the reference
 * does (device_id must exist when use_specific_gpu != 0; otherwise device 0).
 * Empty input (positions_size == 0 or num_patches == 0) returns ADECO_OK.
 */
int adeco_deposit_tets(int use_specific_gpu, size_t device_id, size_t patch_offset, size_t num_patches,
                       const float *positions, size_t positions_size, int meta_cells_per_patch,
                       const float bbox[6], int dims, float *data);

typedef struct {
    int use_specific_gpu;
    size_t device_id;
    size_t patch_offset;
    size_t num_patches;
    const float *positions;      /* host */
    size_t positions_size;       /* floats */
    int meta_cells_per_patch;    /* m */
    const float *bbox;           /* 6 floats */
    int dims;
    void *data;                  /* host grid dims^3, ACCUMULATED, type out_type */
    int out_type;                /* adeco_out_type */
    int precision;               /* adeco_precision */
    int tet_order;               /* adeco_tet_order */
    double tet_mass;             /* mass per tet (reference: 1.0) */
} adeco_deposit_args;

int adeco_deposit_tets_ex(const adeco_deposit_args *args);

/* Device-resident form: positions and the output already in device memory
 * (d_out: FP64 grid, ACCUMULATED), work on `stream` (a cudaStream_t or NULL).
 * Synchronous with respect to the host. */
int adeco_deposit_tets_device(const float *d_positions, size_t positions_size, size_t patch_offset,
                              size_t num_patches, int meta_cells_per_patch, const float bbox[6], int dims,
                              double *d_out, int precision, int tet_order, double tet_mass, void *stream);

/* Same deposit as adeco_deposit_tets_device (mixed precision only) for
 * callers that must not allocate device memory while they deposit: an
 * application that gives all of the GPU's memory to its own pool at start-up
 * (a cudaMalloc inside the deposit would fail, or take memory the pool
 * counts on), or a latency-critical loop where cudaMalloc's unbounded time and
 * cudaFree's device-wide synchronisation are not allowed.
 * No counterpart in the reference (its deposit allocates on every call).
 *
 * Arguments: those of adeco_deposit_tets_device without `precision`.
 * It allocates nothing: its scratch is one fixed device array of 15.5 MB
 * compiled into the library, which every GPU that loads the library holds
 * until the process exits.  Limits, each returning ADECO_ERR_LIMIT:
 * dims^3 <= 96^3 grid cells; num_patches * ceil(m/7)^3 <= 4096 work items;
 * at most max(65536, 256 * work items) ill-conditioned tets (longest edge
 * cubed over |6V| above 32) in one call -- the allocating entry point's
 * limit for the same call.  The first call on a device looks the array up
 * with that device current (cudaGetSymbolAddress); make that first call
 * before any stream capture.  Every call shares the array: calls that
 * overlap on the GPU (other streams or host threads) race and must be
 * serialised.  d_out is ACCUMULATED (+=); the call synchronises `stream`. */
int adeco_deposit_tets_device_noalloc(const float *d_positions, size_t positions_size, size_t patch_offset,
                                      size_t num_patches, int meta_cells_per_patch, const float bbox[6], int dims,
                                      double *d_out, int tet_order, double tet_mass, void *stream);

/* ------------------------------------------------------------------ */
/* Sessions: a resident particle lattice + octree                       */

typedef struct adeco_session adeco_session;

typedef struct {
    int device;             /* CUDA device ordinal                                   */
    int tet_order;          /* adeco_tet_order                                       */
    double tet_mass;        /* mass per tet                                          */
    double hbm_fraction;    /* admission budget: fraction of free HBM (0 -> 0.75)    */
    int accumulate_fp64;    /* 1: sum clipped-piece volumes in FP64 (default 1)      */
} adeco_session_config;

/* positions: host, nx*ny*nz vertices x 3 floats, x fastest (the lattice of
 * particle ids; tets are built from (nx-1)(ny-1)(nz-1) cubes). */
int adeco_session_create(const adeco_session_config *cfg, const float *positions, int nx, int ny, int nz,
                         adeco_session **out);
int adeco_session_destroy(adeco_session *s);

/* Particle file formats: the reference's id_type (src/AdPointDataReaders.h:914-930). */
enum { ADECO_FORMAT_SORTED_BY_ID = 0, ADECO_FORMAT_DARK_SKY = 1 };
/* A session whose lattice is read from a particle file, replacing the
 * reference's reader step of deposit_workflow (src/AdDepositWorkFlow.h:74-111:
 * AdPointDataReader::load_data on one rank, get_global_bbox_mpi,
 * apply_boundary_corrections when periodic != 0).  SORTED_BY_ID: float32
 * x,y,z per particle in id order (AdSortedByIdsPointDataReader, :770;
 * stride ignored, as there).  DARK_SKY: SDF file of {x,y,z,vx,vy,vz float,
 * int64 Morton id} records (AdDarkSkyDataReader, :361), every stride-th
 * particle per axis kept.  bbox_out (may be null): the particles' bounding
 * box before the unwrap -- the reference's global_bbox and default region of
 * interest.  Errors (ADECO_ERR_ARGUMENT): unreadable file, bad header or
 * size, non-cubic lattice, stride not dividing it, ids outside it. */
int adeco_session_create_from_file(const adeco_session_config *cfg, const char *path, int format, int stride,
                                   int periodic, float bbox_out[6], adeco_session **out);
/* lattice size and the resident positions (3 floats per particle, x fastest) */
int adeco_session_lattice_dims(adeco_session *s, int dims[3]);
int adeco_session_positions(adeco_session *s, float *xyz, size_t capacity);
/* particle AABB of the resident lattice: xmin,xmax,ymin,ymax,zmin,zmax */
int adeco_session_bbox(adeco_session *s, float bbox[6]);

typedef struct {
    float min[3];
    float ext;
    int32_t level;
    int32_t parent;
    int32_t first_child;    /* -1 for a leaf */
    int32_t n_meta;         /* meta-cells attached (leaves only) */
    uint64_t estimate;      /* tet-count estimate that drove refinement */
} adeco_node;

/* generate_tree over the resident lattice.  box6 = min xyz, max xyz (NULL:
 * the particle AABB); roi6 likewise (NULL or min > max: the whole box). */
int adeco_session_build_octree(adeco_session *s, const float *box6, const float *roi6,
                               uint64_t max_tets_per_node, int max_level, int leaf_dims);
/* Where adeco_session_build_octree does its per-(node, meta-cell) work: on the
 * device (default) or on the host.  Both give the same tree, node for node. */
enum { ADECO_OCTREE_DEVICE = 0, ADECO_OCTREE_HOST = 1 };
int adeco_session_set_octree_builder(adeco_session *s, int builder);
int adeco_session_octree_size(adeco_session *s, int *n_nodes, int *n_leaves, int *n_levels);
int adeco_session_octree_nodes(adeco_session *s, adeco_node *nodes, int capacity);
/* leaf ids in Octree::getLeafNodes order and each leaf's meta-cell list */
int adeco_session_leaves(adeco_session *s, int32_t *leaf_ids, int capacity);
int adeco_session_leaf_meta(adeco_session *s, int leaf_index, uint64_t *ids, int capacity, int *count);

typedef struct {
    double kernel_ms;       /* device time of the deposit kernels (CUDA events)       */
    double total_ms;        /* device time including conversion                       */
    uint64_t launches;      /* kernel launches made by this call                      */
    uint64_t tets;          /* tets with nonzero volume meeting an output grid        */
    uint64_t candidate_pairs;
    uint64_t partial_pairs;
    uint64_t cell_inside_pairs;
    uint64_t tet_inside_pairs;
    uint64_t fp64_pairs;    /* pairs decided by the FP64 plane test                   */
    uint64_t items;         /* work items (grid x vertex block)                       */
    uint64_t routed_tets;   /* ill-conditioned tets (longest edge^3 > 32 |6V|) that the
                               barycentric route deposited                          */
    uint64_t serial_pieces; /* pieces a lane clipped alone because its warp's piece
                               pool was full and no lane could move (collect_stats) */
} adeco_timing;

/* Deposit every leaf (leaf_dims^3 cells over the leaf's cube) in one batched
 * persistent launch (ADECO_PREC_MIXED) or one FP64 launch per leaf
 * (ADECO_PREC_FP64).  Leaf grids stay on the device; `host_out` (optional)
 * receives n_leaves * leaf_dims^3 FP64 masses in leaf order.  `collect_stats`
 * enables the pair counters (slower; not for timing). */
int adeco_session_deposit_leaves(adeco_session *s, int precision, double *host_out, int collect_stats,
                                 adeco_timing *timing);
/* Device pointer of the FP64 leaf grids of the last deposit (valid until the
 * next deposit or destroy). */
int adeco_session_leaf_grids_device(adeco_session *s, const double **d_grids, size_t *n_values);
/* Capture the batched leaf deposit into a CUDA graph and replay it `reps`
 * times; kernel_ms is the mean device time of one replay. */
int adeco_session_replay_leaves(adeco_session *s, int reps, adeco_timing *timing);

/* Launch-shape and batching parameters of a session's deposits, picked by
 * the project's autotuner (adeco_gb300/tune.py) or set by hand.  Get them,
 * change fields, set them back; out-of-range values return ADECO_ERR_ARGUMENT. */
typedef struct {
    int zoom_tile;           /* cells per tile edge of zoom grids, 16..256 (default 64)              */
    int share_chunk;         /* zoom grids: candidate pairs per work-sharing chunk, 64..8192 (512)  */
    int clip_batch;          /* partial pairs a warp lists before clipping them, 64..128 (128)      */
    int ctas_per_sm;         /* CTAs per SM of the persistent leaf launch, 1..2 (2)                 */
    uint64_t route_capacity; /* ill-conditioned tets one launch may list; more set ADECO_ERR_LIMIT
                                (0: automatic, max(65536, 256 x work items))                         */
    uint32_t item_pairs;     /* zoom grids: a request's tile edge is zoom_tile halved (down to 8)
                                while a work item would hold more expected candidate pairs than this,
                                4096..2^26 (2^18)                                                     */
} adeco_tuning;
int adeco_session_get_tuning(adeco_session *s, adeco_tuning *t);
int adeco_session_set_tuning(adeco_session *s, const adeco_tuning *t);

/* ------------------------------------------------------------------ */
/* Zoom requests, batches and the serving loop                          */

typedef struct {
    float center[3];
    float side;             /* cubic box */
    int dims;               /* cells per axis (multiple of 1, <= 1024) */
    int precision;          /* adeco_precision */
} adeco_request;

/* Queue a batch of requests; returns its id at once.  Continuous batching:
 * a batch is admitted as soon as device memory (a session arena within
 * hbm_fraction of the HBM free at the first submit) and a stream are free,
 * and runs concurrently with the batches already on the GPU, its CTAs taking
 * SMs as theirs finish (cheap batches on higher-priority streams).  Batches
 * that do not fit yet wait inside the library.  ADECO_ERR_MEMORY only when
 * the batch alone exceeds the admission budget. */
int adeco_session_submit(adeco_session *s, const adeco_request *reqs, int n, uint64_t *batch_id);
/* done = 1 when every request of the batch has finished. */
int adeco_session_poll(adeco_session *s, uint64_t batch_id, int *done);
int adeco_session_wait(adeco_session *s, uint64_t batch_id, double timeout_s);
/* FP64 masses of request `index` of a finished batch (dims^3, x fastest). */
int adeco_session_result(adeco_session *s, uint64_t batch_id, int index, double *host_out, size_t capacity);
/* latency (submit -> done, host clock) of request `index`, milliseconds */
int adeco_session_latency(adeco_session *s, uint64_t batch_id, int index, double *ms);
/* device time of the batch's deposit launch (CUDA events on its stream), milliseconds; waits for the batch */
int adeco_session_batch_device_ms(adeco_session *s, uint64_t batch_id, double *ms);
/* Frees the batch's results (host staging), waiting on the host for the
 * batch to finish if it has not; no device-wide synchronisation. */
int adeco_session_release(adeco_session *s, uint64_t batch_id);

typedef struct {
    uint64_t submitted;      /* batches submitted                                          */
    uint64_t completed;      /* batches finished                                           */
    uint64_t queued;         /* batches waiting for memory or a stream now                 */
    uint64_t admission_waits;/* admissions that found no memory or stream free             */
    uint32_t running;        /* batches on the GPU now                                     */
    uint32_t max_running;    /* most batches on the GPU at once                            */
    uint64_t arena_bytes;    /* device memory held by the serving arena                    */
    uint64_t arena_budget;   /* its admission budget                                       */
} adeco_serving_stats;
int adeco_session_serving_stats(adeco_session *s, adeco_serving_stats *st);

/* ------------------------------------------------------------------ */
/* Parity diagnostics (same device functions as the deposit kernels)    */

/* 13 ints per tet of cubes [cube_begin,cube_end) of a patch sequence: the 4
 * corner slots after the orientation rule, volume sign, in-grid flag,
 * candidate range x0,x1,y0,y1,z0,z1, 0.  `cand` (optional, dims^3 uint32,
 * host) receives per cell the number of nonzero-volume tets whose candidate
 * range covers it. */
int adeco_debug_tet_records(const float *positions, size_t positions_size, int meta_cells_per_patch,
                            size_t cube_begin, size_t cube_end, const float bbox[6], int dims, int tet_order,
                            int32_t *records, uint32_t *cand);

/* The bounded wait every spin-wait of the deposit kernels uses, run on a
 * count that nothing decrements, for at most `spins` sleeps of 32 ns: the
 * failure path of a wait that runs out, exercised without a fault.  Returns
 * ADECO_ERR_CUDA with the deposit's "timed out" message (device error bit 3)
 * when the wait ran out, as it must. */
int adeco_debug_bounded_wait(unsigned spins);

/* Measured FP32 FMA throughput of `device` (TFLOP/s, 2 flops per FMA): the
 * peak the deposit kernels' roofline fraction is stated against. */
int adeco_probe_fp32_tflops(int device, double *tflops);

#ifdef __cplusplus
}
#endif
#endif
