/*
 * pma — GB300-native pore-throat and shortest-path pipeline (C ABI).
 *
 * Drop-in for the ImageProcessing services of PorousMediaAnalysis. Every volume-level
 * entry point replaces one service method of the reference; the folder-level entry point
 * replaces the command-line modes. No C++ exceptions cross this boundary: every call
 * returns a pma_status and, on failure, pma_last_error() gives the message (the reference
 * throws Core::InvalidOperationException and prints it in Main.cpp:62-98).
 *
 * Volumes are dense arrays in the reference's memory order [z][x][y] (y fastest,
 * DataArray.h:85-94): x is the TIFF row, y the TIFF column, z the slice. Device pointers
 * are plain CUDA device addresses on the context's device. Element types are those of
 * ImageProcessing/Model/Headers/Types.h:16-25 (uint32 for squared distances, ids and
 * coordinates; uint8 masks; float32 geodesics, plus a float64 variant).
 *
 * The total voxel count of one volume must stay below 2^32.
 */
#ifndef PMA_H
#define PMA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PMA_ABI_VERSION 1

typedef enum pma_status {
    PMA_OK = 0,
    PMA_ERR_ARGUMENT = 1,   /* bad size, null pointer, unsupported option */
    PMA_ERR_CUDA = 2,       /* CUDA runtime error or missing device */
    PMA_ERR_IO = 3,         /* file missing, unreadable or malformed */
    PMA_ERR_MEMORY = 4,     /* device or host allocation failed, or budget exceeded */
    PMA_ERR_LIMIT = 5,      /* a bounded device loop gave up (iteration limit reached) */
    PMA_ERR_INTERNAL = 6
} pma_status;

typedef struct pma_dims {
    int32_t sx, sy, sz;     /* X (rows), Y (columns), Z (slices) */
} pma_dims;

/* Stencil of pore propagation, watershed and geodesics ("Use D3Q7 stencil", Config.h:39). */
typedef enum pma_stencil { PMA_D3Q27 = 0, PMA_D3Q7 = 1 } pma_stencil;

/* Copies the calling thread's last error message into buf; returns its full length. */
size_t pma_last_error(char* buf, size_t cap);
int pma_abi_version(void);

/* ---------------------------------------------------------------------------------
 * Context: one device, one CUDA stream, cached device scratch memory.
 * ------------------------------------------------------------------------------- */
typedef struct pma_ctx pma_ctx;
int pma_ctx_create(int device, pma_ctx** out);
int pma_ctx_destroy(pma_ctx* ctx);
/* Runs subsequent work of ctx on an existing cudaStream_t (NULL = a new stream of the
 * context's own; pass cudaStreamLegacy to share the legacy default stream). */
int pma_ctx_set_stream(pma_ctx* ctx, void* cuda_stream);
/* Number of this library's kernels launched through ctx (and its batch lanes) since creation. */
uint64_t pma_ctx_launch_count(const pma_ctx* ctx);
/* Opt-in kernel timing: with timing on, the hot kernels are bracketed by CUDA events on
 * the context's stream. The report is a JSON object {"kernel": [total_ms, launches], ...}
 * of everything timed since the previous report; each call consumes the timed events, so
 * pass a buffer large enough for the whole report. Returns its full length. Work counters
 * of the timed calls appear as "count.<name>": [sum, increments]. */
int pma_ctx_set_timing(pma_ctx* ctx, int enable);
size_t pma_ctx_timing_report(pma_ctx* ctx, char* buf, size_t cap);
/* Bounds of the data-dependent device loops. Each loop that reaches its bound stops and the
 * call returns PMA_ERR_LIMIT, with the context still usable. No counterpart in the
 * reference, whose loops run on the host; the defaults are far above what any volume of
 * fewer than 2^32 voxels needs. Batch lanes and server lanes created later inherit them. */
typedef struct pma_limits {
    int32_t spin_limit;             /* polls of one device-side wait on another block (2^20) */
    int32_t union_limit;            /* link attempts of one plateau union in the union-find (2^22) */
    uint64_t watershed_generations; /* FIFO generations of one watershed call (2^23 - 1) */
    uint64_t geodesic_buckets;      /* distance buckets of one cavity's flood (0: 2 * voxels + 64) */
} pma_limits;
int pma_ctx_get_limits(const pma_ctx* ctx, pma_limits* out);
int pma_ctx_set_limits(pma_ctx* ctx, const pma_limits* limits);
/* Shared-type numbering of pma_pores: 0 (default) an order that matches the reference's up
 * to a renaming, 1 the reference's creation order (a host replay; see pma_pores). Batch and
 * server lanes created later inherit it. pma_run_folder always uses the reference's. */
int pma_ctx_set_throat_numbering(pma_ctx* ctx, int reference_order);
/* Runs the bounded device waits on a flag that nothing sets (both forms of the watershed's
 * frontier look-back waiting for a chunk that never publishes), with the context's spin_limit.
 * Sets *timed_out = 1 when every wait gave up and reported it, as it must. No counterpart in the
 * reference; it exercises the error path of the device waits without faulting anything. */
int pma_selftest_bounded_wait(pma_ctx* ctx, int* timed_out);

/* Device bytes held by ctx's scratch cache and its memory pool (freed blocks are kept for
   reuse), batch lanes included; pma_ctx_trim releases them. */
size_t pma_ctx_scratch_bytes(const pma_ctx* ctx);
int pma_ctx_trim(pma_ctx* ctx);

/* ---------------------------------------------------------------------------------
 * Stage entry points on device buffers. All run on the context's stream and return
 * after the stream work they need on the host has completed.
 * ------------------------------------------------------------------------------- */

typedef struct pma_edt_stats {
    uint32_t max_edt2;          /* "Max Euclidean distance square" */
    uint32_t pad_;
    uint64_t hist_len;          /* max_edt2 + 1 */
} pma_edt_stats;

/* Squared Euclidean distance transform, its maximum and the histogram of balls that do
 * not cross the image boundary. Replaces EuclideanDistanceComputer::ComputeEuclideanDistances
 * (EuclideanDistanceComputer.cpp:30-44; passes :149-343). d_solid: non-zero = solid.
 * h_hist (host, may be NULL) receives min(hist_cap, max_edt2+1) counters. */
int pma_edt(pma_ctx* ctx, const uint8_t* d_solid, pma_dims dims, uint32_t* d_edt2,
            pma_edt_stats* stats, uint64_t* h_hist, size_t hist_cap);

/* Allocation-free variant of pma_edt. No counterpart in the reference: it gives the same
 * results as pma_edt (EuclideanDistanceComputer.cpp:30-44) for callers that cannot let
 * the library allocate device memory. It takes no context, calls no allocator and runs
 * on the calling thread's current device, on cuda_stream (NULL = the legacy default
 * stream); it returns once that stream's work for the call is complete.
 * Its only scratch, the histogram bins and the maximum, is a fixed array of
 * PMA_EDT_NOALLOC_MAX_HIST_BINS 64-bit counters (2 MiB) in the library's global memory,
 * cleared by every call. Volumes whose smallest extent is above 1024 need more bins and
 * are rejected with PMA_ERR_LIMIT.
 * The first call on a device looks up the scratch address on that device (set-up); make
 * that first call before any stream capture. All calls on one device share the scratch:
 * calls that overlap in time (from several host threads, or on streams not ordered with
 * each other) race on it and return wrong statistics. */
#define PMA_EDT_NOALLOC_MAX_HIST_BINS 262144
int pma_edt_noalloc(const uint8_t* d_solid, pma_dims dims, uint32_t* d_edt2,
                    pma_edt_stats* stats, uint64_t* h_hist, size_t hist_cap, void* cuda_stream);

/* Containing-ball radii (squared), the winning centre of each void voxel and the
 * IsMaximumBall mask (0 solid, 127 inner, 255 outer). Replaces
 * ContainingBallsAssigner::SetContainingBalls (ContainingBallsAssigner.cpp:36-60;
 * scatter :101-183, mask :190-250) with its single-thread tie rule: the winner is the
 * lexicographically smallest (x, y, z) centre among those of maximal radius. */
int pma_containing_balls(pma_ctx* ctx, const uint32_t* d_edt2, pma_dims dims, uint32_t max_edt2,
                         uint32_t* d_crad2, uint32_t* d_cx, uint32_t* d_cy, uint32_t* d_cz,
                         uint8_t* d_maxball_mask, uint64_t* h_maximum_balls_count);

/* Pores and throats table (host memory, owned by the library). */
typedef struct pma_pore {       /* a row of pores.txt (Serializer.cpp:187-201) */
    uint32_t id;
    int32_t seed_x, seed_y, seed_z;
    uint32_t seed_r2;
    int32_t is_boundary;
    uint64_t volume;
} pma_pore;

typedef struct pma_throat {     /* a row of sharedPixelTypes.txt (Serializer.cpp:203-221) */
    uint32_t id;
    uint32_t n_pores;
    uint64_t volume;
    uint64_t pool_offset;       /* pore ids at pool[pool_offset .. pool_offset + n_pores) */
} pma_throat;

typedef struct pma_table pma_table;
int pma_table_create(const pma_pore* pores, size_t n_pores, const pma_throat* throats,
                     size_t n_throats, const uint32_t* pool, size_t pool_size, pma_table** out);
size_t pma_table_npores(const pma_table* t);
const pma_pore* pma_table_pores(const pma_table* t);
size_t pma_table_nthroats(const pma_table* t);
const pma_throat* pma_table_throats(const pma_table* t);
size_t pma_table_pool_size(const pma_table* t);
const uint32_t* pma_table_pool(const pma_table* t);
void pma_table_free(pma_table* t);

/* Pore seeds and the initial pore propagation: replaces
 * PoreAndThroatComputer::AssignPoreAndThroatIds (PoreAndThroatComputer.cpp:35-55; seeds
 * :93-163, propagation :192-269, pixel states BasePoreAndThroatComputer.cpp:37-133).
 * Pore ids, seeds, radii, volumes, boundary flags and every voxel's pore set are exact.
 * Shared-type ("throat") ids count down from UINT32_MAX - 1. By default they are numbered
 * in order of (last pore of the type, first voxel of the type): the reference's types and
 * labels up to a one-to-one renaming of the type ids. After
 * pma_ctx_set_throat_numbering(ctx, 1) they are the reference's own ids: the order in which
 * its depth-first searches create the types (types deleted later included), reproduced by
 * a host replay of each pore's search order. That replay is sequential per pore and costs
 * about one visit per voxel of every pore's reach set (tens of seconds at 1024^3), so the
 * folder-level entry point uses it (it writes these ids into PoreThroatIds and
 * sharedPixelTypes.txt) and the other entry points leave it to the caller. Nothing
 * downstream of the empty-pore removal depends on the numbering (the watershed reads only
 * the pores). d_labels is written completely. */
int pma_pores(pma_ctx* ctx, const uint8_t* d_maxball_mask, const uint32_t* d_edt2,
              const uint32_t* d_crad2, pma_dims dims, pma_stencil stencil, uint32_t* d_labels,
              pma_table** out);

/* Drops zero-volume pores, merges and renames throats and remaps d_labels. Replaces
 * EmptyPoresRemover::RemoveEmptyPores (EmptyPoresRemover.cpp:31-244). */
int pma_remove_empty_pores(pma_ctx* ctx, pma_table* table, uint32_t* d_labels, pma_dims dims);

/* Watershed labelling from the pores of `pores`. Replaces
 * WatershedComputer::AssignPoreAndThroatIds (WatershedComputer.cpp:30-219), bit-exact
 * including throat ids. d_labels_ws is written completely. */
int pma_watershed(pma_ctx* ctx, const pma_table* pores, const uint32_t* d_crad2, pma_dims dims,
                  pma_stencil stencil, uint32_t max_edt2, uint32_t* d_labels_ws, pma_table** out);

typedef struct pma_cavity {     /* a row of cavityDescriptions.txt (Serializer.cpp:161-185) */
    uint32_t id;
    int32_t seed_x, seed_y, seed_z;
    float distance_to_center;
    int32_t reached_walls;
    uint64_t void_count;
    int32_t reaches_all_walls;
    int32_t pad_;
} pma_cavity;

/* Geodesic distances from the void voxel nearest the centre, cavity restarts and cavity
 * ids. Replaces ShortestPathComputer::ComputeShortestPathDistances
 * (ShortestPathComputer.cpp:39-511). Distances: -1 solid, FLT_MAX (DBL_MAX) unreached;
 * cavity ids: 0 solid, UINT32_MAX unreached. The f32 variant is bit-exact with the
 * reference; the f64 variant accumulates the same steps in double precision.
 * Cavity rows (cavityDescriptions.txt, ShortestPathComputer.cpp:143-164): the first
 * cavity_cap rows are written to h_cavities and *n_cavities receives the number of
 * cavities, which may exceed cavity_cap (call again with a larger buffer to get them all;
 * cavity_cap 0 with h_cavities NULL only counts). */
int pma_geodesic_f32(pma_ctx* ctx, const uint8_t* d_solid, pma_dims dims, pma_stencil stencil,
                     float* d_dist, uint32_t* d_cavity, pma_cavity* h_cavities, int cavity_cap,
                     int* n_cavities);
int pma_geodesic_f64(pma_ctx* ctx, const uint8_t* d_solid, pma_dims dims, pma_stencil stencil,
                     double* d_dist, uint32_t* d_cavity, pma_cavity* h_cavities, int cavity_cap,
                     int* n_cavities);

/* ---------------------------------------------------------------------------------
 * Whole pipeline on one volume, host buffers in and out (EDT -> containing balls ->
 * pores -> empty-pore removal -> watershed, plus geodesics), the host<->device copies
 * included. Any output pointer may be NULL to skip copying that field back. Page-locked
 * buffers (cudaHostAlloc, cudaHostRegister) are read and written by a streaming kernel
 * through their mapped address, at the link's full rate; pageable ones through
 * cudaMemcpyAsync.
 * ------------------------------------------------------------------------------- */
typedef struct pma_outputs {
    uint32_t* edt2;             /* EuclideanDistanceSquares */
    uint32_t* crad2;            /* ContainingBallRadiiSquares */
    uint32_t* cx; uint32_t* cy; uint32_t* cz;   /* ContainingBallCoordinatesX/Y/Z */
    uint8_t* maxball_mask;      /* IsMaximumBall */
    uint32_t* pore_labels;      /* PoreThroatIds (after empty-pore removal) */
    uint32_t* watershed_labels; /* PoreThroatIdsWatershed */
    float* dist_f32;            /* ShortestPathDistances, float32 (geodesic_fp64 = 0) */
    double* dist_f64;           /* geodesics in float64 (geodesic_fp64 = 1) */
    uint32_t* cavity;           /* CavityIds */
    /* results filled by the call */
    pma_edt_stats edt_stats;
    uint64_t maximum_balls_count;
    pma_table* pores;           /* after empty-pore removal (caller frees) */
    pma_table* watershed;       /* watershed pores and throats (caller frees) */
    pma_cavity cavities[16];    /* the first 16 cavity rows */
    int n_cavities;             /* the number of cavities (may exceed 16) */
    int cavity_rows_cap;        /* capacity of cavity_rows */
    pma_cavity* cavity_rows;    /* optional host buffer: receives the first cavity_rows_cap rows */
} pma_outputs;

typedef struct pma_options {
    pma_stencil stencil;
    int run_pores;              /* 1: EDT..watershed */
    int run_geodesic;           /* 1: geodesics */
    int geodesic_fp64;          /* 1: geodesics in float64 only (dist_f64), 0: float32 */
} pma_options;

int pma_pipeline_host(pma_ctx* ctx, const uint8_t* h_solid, pma_dims dims,
                      const pma_options* opts, pma_outputs* out);

/* ---------------------------------------------------------------------------------
 * Batched form: many independent volumes of uneven sizes in one call. No counterpart in
 * the reference, which processes sample folders one after another
 * (CommandLineDispatcher.cpp:62-71).
 * ------------------------------------------------------------------------------- */
typedef struct pma_batch_item {
    const uint8_t* solid;       /* [z][x][y] volume, non-zero = solid: host memory, or
                                   device memory when the call is resident */
    pma_dims dims;
    int status;                 /* set by the call: this volume's pma_status */
    pma_outputs* out;           /* as for pma_pipeline_host; with resident = 1 its field
                                   pointers are device pointers (NULL = not kept) */
} pma_batch_item;

/* Runs the whole chain (options as pma_pipeline_host) on n volumes with up to `lanes` of them
 * in flight at once (0 = 8, at most 64), each lane with its own stream, host thread and
 * scratch memory, kept by ctx for later calls. Every volume's results equal a separate
 * pma_pipeline_host call. Returns PMA_OK when all volumes succeeded, else the status of the
 * first failing one (pma_last_error names it); the other volumes still complete. */
int pma_pipeline_batch(pma_ctx* ctx, pma_batch_item* items, size_t n, const pma_options* opts,
                       int resident, int lanes);

/* ---------------------------------------------------------------------------------
 * Serving: a request loop with continuous batching under a device-memory budget. No
 * counterpart in the reference. Requests are admitted in arrival order as lanes (child
 * contexts with their own stream, scratch and host thread) and budget free up; requests in
 * flight overlap on the device, and each request's fields stay on the device from the first
 * stage to the last. Every result equals a separate pma_pipeline_host call.
 * ------------------------------------------------------------------------------- */
typedef struct pma_server pma_server;

typedef struct pma_server_config {
    int lanes;                  /* requests in flight at most (0 = 8, at most 64) */
    int pad_;
    uint64_t memory_budget;     /* device bytes for all lanes' fields and scratch (0 = 120 GiB) */
    pma_options options;        /* as for pma_pipeline_host */
} pma_server_config;

typedef struct pma_server_stats {
    uint64_t submitted, completed, failed, rejected;
    uint64_t queued;
    uint64_t peak_reserved_bytes;   /* largest sum of lane reservations at an admission */
    uint64_t resident_bytes;        /* lanes' device scratch now */
    double bytes_per_voxel;         /* footprint estimate used for admission */
    uint32_t max_in_flight;
    uint32_t pad_;
} pma_server_stats;

int pma_server_create(pma_ctx* ctx, const pma_server_config* cfg, pma_server** out);
/* Queues one volume (host memory, [z][x][y], non-zero = solid); h_solid and out (host output
 * buffers and tables as for pma_pipeline_host) must stay valid until the request completes. */
int pma_server_submit(pma_server* srv, const uint8_t* h_solid, pma_dims dims, pma_outputs* out,
                      uint64_t* ticket);
/* Waits for a request (timeout_ms < 0: no limit; PMA_ERR_LIMIT when it runs out) and
 * returns PMA_OK with *status = the request's own status (PMA_ERR_MEMORY if it alone exceeds
 * the budget) and its latency from submission to completion. A ticket is waited for once. */
int pma_server_wait(pma_server* srv, uint64_t ticket, int64_t timeout_ms, int* status,
                    double* latency_ms);
int pma_server_get_stats(pma_server* srv, pma_server_stats* out);
/* Completes the queued requests, then releases the lanes. */
int pma_server_destroy(pma_server* srv);

/* ---------------------------------------------------------------------------------
 * Folder-level drop-in for the command-line modes (CommandLineDispatcher.cpp:34-72,
 * ImageProcessingManager.cpp:63-108): walks every folder under base_folder holding a
 * config.txt, reads Images/ and writes the same TIFF folders and text files.
 * ------------------------------------------------------------------------------- */
typedef enum pma_mode {
    PMA_MODE_ALL = 1, PMA_MODE_EDT = 2, PMA_MODE_RIB = 3, PMA_MODE_APT = 4, PMA_MODE_SPD = 5
} pma_mode;

int pma_run_folder(pma_ctx* ctx, const char* base_folder, pma_mode mode);

/* ---------------------------------------------------------------------------------
 * Host I/O (no GPU needed).
 * ------------------------------------------------------------------------------- */
/* Reads a TIFF stack folder (slices sorted by name) of 1- or 4-byte voxels into
 * [z][x][y]. With out == NULL only dims are filled. */
int pma_read_tiff_stack(const char* folder, int bytes_per_voxel, pma_dims* dims, void* out,
                        size_t out_bytes);
/* Writes [z][x][y] voxels as slices 1.tif .. SZ.tif, zero-padded to the width of SZ so
 * that the name order is the slice order (8-bit grey or 32-bit CMYK LZW). */
int pma_write_tiff_stack(const char* folder, int bytes_per_voxel, pma_dims dims, const void* data);

/* The run configuration of a sample folder. Replaces Serializer::ReadConfig
 * (Serializer.cpp:31-64): the same five lines in the same fscanf format, the resolutions
 * divided by the smallest one. Unlike the reference, which keeps -1 in fields that do not
 * parse, a file whose first four lines do not parse, or whose resolutions are not
 * positive, is rejected with PMA_ERR_IO. */
typedef struct pma_run_config {
    double resolution[3];       /* "Resolution of initial images", normalised (smallest = 1) */
    double max_pore_radius_ratio;
    int32_t available_memory_mb;
    int32_t use_d3q7;
    int32_t threads;            /* -1 when the line is missing */
    int32_t pad_;
} pma_run_config;
int pma_read_config(const char* path, pma_run_config* out);

#ifdef __cplusplus
}
#endif
#endif /* PMA_H */
