/*
 * gp_ptp.h -- C ABI of the GB300-native Parallel Toplesets Propagation (PTP)
 * geodesics library (libgp_ptp.so).
 *
 * This is the drop-in boundary for gproshan's PTP_GPU path.  Every entry point
 * takes plain pointers and sizes, returns a gp_status, never calls
 * cudaDeviceReset and never aborts the process.  Each one lists the reference
 * interface it replaces (paths are inside the gproshan source tree).
 *
 * Types follow the reference: index_t = uint32_t, NIL = 0xFFFFFFFF
 * (include/include.h:12,19).  Distances are float (the reference's SINGLE_P
 * build) or double (its default build); the caller picks per call.
 *
 * Threading: one gp_ctx per thread (a context owns one CUDA stream and a
 * workspace); meshes belong to the context that made them.  Calls on one
 * context are serialised by the caller.
 */
#ifndef GP_PTP_H
#define GP_PTP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GP_NIL 0xFFFFFFFFu
#define GP_PTP_TOL 1e-3 /* PTP_TOL, include/geodesics_ptp.h:11 */

typedef enum gp_status {
	GP_OK = 0,
	GP_ERR_INVALID_ARG = 1,     /* null pointer, size out of range, bad vertex index */
	GP_ERR_NONMANIFOLD = 2,     /* a star walk does not close within the mesh size */
	GP_ERR_NO_CONVERGENCE = 3,  /* reserved: the reference stops at max_iter silently */
	GP_ERR_DEVICE_TIMEOUT = 4,  /* a device-side wait ran past its limit */
	GP_ERR_CUDA = 5,            /* a CUDA runtime call failed; see gp_ctx_last_error */
	GP_ERR_NO_DEVICE = 6,       /* no CUDA device / not an sm_103 device */
	GP_ERR_OUT_OF_MEMORY = 7,
	GP_ERR_CAPACITY = 8         /* an output buffer is too small */
} gp_status;

typedef enum gp_dtype { GP_F32 = 0, GP_F64 = 1 } gp_dtype;

typedef struct gp_ctx gp_ctx;
typedef struct gp_mesh gp_mesh;

/* ------------------------------------------------------------------ */
/* context                                                             */
/* ------------------------------------------------------------------ */

/* Create a context on CUDA device `device` (one stream, one workspace).
 * Replaces the per-call cudaDeviceReset + cudaMalloc of
 * src/cuda/geodesics_ptp.cu:22-46 with a reusable workspace. */
gp_status gp_ctx_create(int device, gp_ctx **out);
void gp_ctx_destroy(gp_ctx *ctx);
/* 1 if the context's device handles are still usable, 0 if the device was
 * reset since the context was made (cudaDeviceReset destroys the CUDA context
 * they belong to: gproshan's heat-flow code resets the device on every call,
 * src/cuda/heat_flow.cu:47).  A dead context can only be destroyed (which then
 * frees host memory only); meshes made in it are dead too.  No reference
 * counterpart. */
int gp_ctx_valid(const gp_ctx *ctx);
/* Text of the last error seen by this context ("" if none). */
const char *gp_ctx_last_error(const gp_ctx *ctx);
const char *gp_status_str(gp_status s);
/* The context's cudaStream_t, as void*. */
void *gp_ctx_stream(gp_ctx *ctx);
/* Bytes of device workspace currently held by the context. */
size_t gp_ctx_workspace_bytes(const gp_ctx *ctx);
/* The context's device and the code loaded for it: compute capability
 * (10 * major + minor), the binary version of the sweep kernel's loaded code
 * (cudaFuncGetAttributes; 103 = native sm_103 code, not JIT from PTX) and the
 * number of SMs.  Any pointer may be null.  No reference counterpart. */
gp_status gp_ctx_device_info(const gp_ctx *ctx, int *compute_capability, int *binary_version, int *num_sms);

/* ------------------------------------------------------------------ */
/* mesh                                                                */
/* ------------------------------------------------------------------ */

/* Host-side compact half-edge build: opposite table OT[3*n_faces] and extra
 * vertex table EVT[n_vertices] from VT[3*n_faces], with the reference's
 * matching and non-manifold rules (che::update_evt_ot_et, src/che.cpp:1295-1362).
 * *manifold (may be null) receives 1 or 0. */
gp_status gp_che_build(uint32_t n_vertices, uint32_t n_faces, const uint32_t *VT,
                       uint32_t *OT, uint32_t *EVT, int *manifold);

/* Upload a CHE mesh (host arrays: xyz[3*n_vertices], VT/OT[3*n_faces],
 * EVT[n_vertices]) and build its device star lists.  Coordinates are kept as
 * float (FP32 path) and double (FP64 path).  OT/EVT may be null, in which case
 * they are built with gp_che_build.
 * Replaces cuda_create_CHE (src/cuda/che.cu:29-48) and CHE::CHE
 * (src/che.cpp:36-46). */
gp_status gp_mesh_create(gp_ctx *ctx, uint32_t n_vertices, const double *xyz,
                         uint32_t n_faces, const uint32_t *VT, const uint32_t *OT,
                         const uint32_t *EVT, gp_mesh **out);
void gp_mesh_destroy(gp_mesh *mesh);
uint32_t gp_mesh_n_vertices(const gp_mesh *mesh);
uint32_t gp_mesh_n_faces(const gp_mesh *mesh);

/* ------------------------------------------------------------------ */
/* toplesets                                                           */
/* ------------------------------------------------------------------ */

/* Multi-source BFS over the mesh's directed link relation, on the GPU.
 * rings[n_vertices]: ring index per vertex (NIL if unreached);
 * sorted[cap_sorted]: vertices in BFS order (sources repeat if given twice);
 * limits[cap_limits]: start of each ring, then the end.  Output equals
 * che::compute_toplesets bit for bit (src/che.cpp:546-593, link at 102-112).
 * Host buffers; any of rings/sorted may be null. */
gp_status gp_toplesets(gp_ctx *ctx, gp_mesh *mesh, const uint32_t *sources, uint32_t n_sources,
                       uint32_t *rings, uint32_t *sorted, uint32_t cap_sorted,
                       uint32_t *limits, uint32_t cap_limits, uint32_t *n_limits);

/* ------------------------------------------------------------------ */
/* PTP                                                                 */
/* ------------------------------------------------------------------ */

typedef struct gp_ptp_opts {
	uint32_t precision;    /* GP_F32 (closed-form FP32 update) or GP_F64 (reference formula) */
	uint32_t max_iter;     /* 0: the reference's 2*|limits| (src/cuda/geodesics_ptp.cu:204) */
	double tol;            /* 0: PTP_TOL */
	uint32_t threads;      /* reserved (threads per CTA are fixed per kernel) */
	uint32_t ctas;         /* CTAs of the grid-wide launch, 0: all that fit */
	uint32_t local_window; /* fields whose windows stay within this many vertices are
	                          swept by one CTA each; 0: default (GP_F32: 4096, GP_F64: 256) */
	uint32_t round_coords; /* GP_F64 only: 1 = solve on the float-rounded coordinates
	                          the GP_F32 path sees (an FP64 check of an FP32 run) */
	uint32_t schedule;     /* GP_SCHED_REACTIVE (0) or GP_SCHED_LEARNED (1): see below */
	uint32_t grid_kernel;  /* GP_GRID_AUTO (0), GP_GRID_LOCKSTEP (1) or GP_GRID_QUEUE (2) */
	uint32_t queue_min;    /* GP_GRID_AUTO: the work queue when at least this many fields
	                          reach the grid-wide sweeps; 0: default */
	uint32_t queue_tile;   /* work queue: window vertices per claimed tile (a multiple of
	                          32, at most 1024); 0: chosen per window */
	uint32_t normalize;    /* 1: every field's output divided by its largest finite
	                          distance, as normalize_ptp does (src/geodesics_ptp.cpp:
	                          264-276; geodesics::normalize, src/geodesics.cpp:78-90),
	                          on the device before any copy out: the maximum is
	                          reduced inside the output gather */
	uint32_t stream_min;   /* GP_F32 without labels, lockstep grid launch: fields on meshes
	                          of at least this many vertices (and at most 7 fan entries
	                          per vertex) build their toplesets inside the sweep launch,
	                          whose sweeps start as soon as the first rings are ready;
	                          same results.  0: the default, 2^18 in calls of more than
	                          8 fields, never in smaller calls (their large fields build
	                          toplesets with the whole GPU first); 0xFFFFFFFF: never */
} gp_ptp_opts;

/* Grid-wide sweeps of the fields that outgrow one CTA.  LOCKSTEP: one
 * cooperative launch, one sweep of every live field per step, a grid barrier
 * between steps.  QUEUE: one persistent launch whose warps claim tiles of any
 * field with work; a field's next sweep opens as soon as its own sweep is
 * complete (no grid barrier).  Same sweeps, same results. */
#define GP_GRID_AUTO 0u
#define GP_GRID_LOCKSTEP 1u
#define GP_GRID_QUEUE 2u

/* Batch scheduling.  REACTIVE: every field starts on one CTA and moves to the
 * grid-wide launch when a window outgrows local_window.  LEARNED: the context's
 * cost model (gp_ctx_set_cost_model) predicts each field's sweeps and work from
 * its toplesets; fields expected to outgrow one CTA start on the grid launch,
 * the rest are taken longest-predicted-first.  Results are identical. */
#define GP_SCHED_REACTIVE 0u
#define GP_SCHED_LEARNED 1u

typedef struct gp_ptp_stats {
	uint32_t n_iter;       /* sweeps run */
	uint32_t n_limits;     /* |limits| of the toplesets used */
	uint64_t relaxations;  /* vertex relaxations (sum of window sizes) */
	double seconds;        /* device time of the call (CUDA events) */
} gp_ptp_stats;

/*
 * Geodesic distances from `sources` (host array).
 *
 * toplesets: limits/sorted as che::compute_toplesets returns them (host
 * arrays), or both null to build them on the GPU.
 * dist: host array of n_vertices elements of type dist_type; unreached
 * vertices get INFINITY.  clusters (may be null): host array of n_vertices
 * labels; on entry it holds the initial labels, on return source k's region
 * carries k+1 (GPU rule, src/cuda/geodesics_ptp.cu:257-282).
 *
 * Replaces parallel_toplesets_propagation_gpu (src/cuda/geodesics_ptp.cu:20-85)
 * and parallel_toplesets_propagation_coalescence_gpu
 * (src/cuda/geodesics_ptp_coalescence.cu:21-100): the result is the buffer
 * the last sweep wrote, as those return.
 */
gp_status gp_ptp(gp_ctx *ctx, gp_mesh *mesh, const uint32_t *sources, uint32_t n_sources,
                 const uint32_t *limits, uint32_t n_limits, const uint32_t *sorted,
                 const gp_ptp_opts *opts, void *dist, gp_dtype dist_type,
                 uint32_t *clusters, gp_ptp_stats *stats);

/* One field of a batch. */
typedef struct gp_field {
	gp_mesh *mesh;
	const uint32_t *sources;   /* n_sources vertex ids */
	uint32_t n_sources;
	void *dist;                /* n_vertices outputs of the batch's dist_type */
	uint32_t *clusters;        /* null or n_vertices labels (in/out) */
	gp_ptp_stats *stats;       /* null or per-field statistics */
} gp_field;

#define GP_BATCH_DEVICE_POINTERS 1u /* sources/dist/clusters are device pointers */

/*
 * Many independent fields (any meshes, any source sets) solved together: the
 * GPU toplesets of every field, then one persistent launch that sweeps the
 * windows of all live fields each step.  Each field's result equals what
 * gp_ptp returns for it alone.  No reference counterpart: the reference runs
 * one field per call (src/cuda/geodesics_ptp.cu:20).
 */
gp_status gp_ptp_batch(gp_ctx *ctx, const gp_field *fields, uint32_t n_fields,
                       const gp_ptp_opts *opts, gp_dtype dist_type, uint32_t flags,
                       double *seconds);

/* Device timings and counts of the last gp_ptp / gp_ptp_batch / gp_toplesets
 * call on a context (CUDA events between the phases, on the context's stream).
 * No reference counterpart: the reference times a whole call with one event
 * pair (src/cuda/geodesics_ptp.cu:24-84). */
typedef struct gp_call_stats {
	uint32_t launches;         /* kernels this library launched in the call */
	uint32_t n_fields;
	uint32_t fields_grid;      /* fields swept by the grid-wide launch */
	uint32_t sweeps_grid;      /* steps of the lockstep launch, or sweeps completed by the queue launch */
	uint32_t grid_kernel;      /* GP_GRID_LOCKSTEP, GP_GRID_QUEUE, or 0 if no field reached it */
	uint32_t fields_streamed;  /* fields whose toplesets the lockstep launch built (gp_ptp_opts::stream_min) */
	double ms_toplesets;       /* BFS setup + BFS */
	double ms_renumber;        /* ring renumbering passes */
	double ms_local;           /* classify + one-CTA-per-field sweeps */
	double ms_grid;            /* grid-wide persistent sweeps */
	double ms_gather;          /* output gather */
	uint64_t relax_local;      /* vertex relaxations done by the one-CTA launch */
	uint64_t relax_grid;       /* vertex relaxations done by the grid-wide launch */
	uint64_t h2d_bytes;        /* host -> device bytes copied by the call */
	uint64_t d2h_bytes;        /* device -> host bytes copied by the call */
	uint64_t skip_grid;        /* relaxations of the lockstep launch whose inputs were unchanged since the
	                              previous sweep (FP32 without labels): solves skipped, same result */
} gp_call_stats;

gp_status gp_ctx_call_stats(const gp_ctx *ctx, gp_call_stats *out);

/* Step trace of the grid-wide sweep launch.  With out == null: arm the trace
 * for up to cap steps of the following calls (cap = 0 disarms).  Otherwise
 * copy the last call's trace: 2 words per step, the step's start time (ns,
 * device global timer) and (tiles << 32 | live fields); *n_out = steps.
 * Used to study and learn the sweep schedule.  No reference counterpart (the
 * reference writes a per-iteration "band" file in its test harness,
 * src/cuda/test_geodesics_ptp_coalescence.cu:214-266). */
gp_status gp_ctx_step_trace(gp_ctx *ctx, uint32_t cap, uint64_t *out, uint32_t *n_out);

/*
 * gp_toplesets without any device allocation, for callers that may not
 * allocate device memory while they work: an application that handed all
 * device memory to its own pool up front, or a latency-critical loop in which
 * cudaMalloc / cudaFree (which can stall the whole device) are not allowed.
 * It has no counterpart in the reference: the results are gp_toplesets' (the
 * toplesets rings, sorted order and limits), written to caller-provided
 * DEVICE buffers.
 *
 * The BFS scratch (8 bytes per vertex plus a 4 KiB descriptor) is a fixed
 * array inside the library, about 8 MiB, reserved on every GPU that loads the
 * library until the process exits; meshes above 2^20 vertices get
 * GP_ERR_CAPACITY.  The mesh's device must be current.  Every call made
 * outside stream capture looks up the array's device address
 * (cudaGetSymbolAddress), so a device reset between calls is harmless; a call
 * made while its stream is being captured reuses the address found by the
 * last uncaptured call on that device, so the first call on a device (and the
 * first after a device reset) must come before any capture, else the call
 * returns GP_ERR_INVALID_ARG.  Work is enqueued on `stream` (a cudaStream_t,
 * 0 = default stream) and the call returns without waiting.  All calls share
 * the one array, which keeps the last call's contents (each call clears what
 * must start at zero): calls that overlap on the GPU (other streams, other
 * threads) race and must be serialised by the caller.
 *
 * sources: device array of n_sources vertex ids.  rings[n_vertices],
 * sorted[cap_sorted >= n_vertices + n_sources], limits[cap_limits >=
 * n_vertices + 2]: device outputs as gp_toplesets writes them.  *n_limits
 * (device word) receives |limits|, or 0 if a source is out of range.
 */
gp_status gp_toplesets_noalloc(const gp_mesh *mesh, const uint32_t *sources, uint32_t n_sources,
                               uint32_t *rings, uint32_t *sorted, uint32_t cap_sorted, uint32_t *limits,
                               uint32_t cap_limits, uint32_t *n_limits, void *stream);

/* ------------------------------------------------------------------ */
/* learned sweep-cost model                                            */
/* ------------------------------------------------------------------ */
/*
 * A 3-layer MLP (GP_MLP_IN -> 64 -> 64 -> 2, ReLU) predicting, per field,
 * log(sweeps / rings) and log(relaxations / vertices) from the field features
 * of gp_field_features.  Trained on the GPU by the library's own FP32
 * forward/backward/Adam kernels; evaluated with BF16 tensor-core inference.
 * It only steers scheduling (where a field starts, the order fields are taken);
 * results never depend on it.  No reference counterpart: gproshan runs a fixed
 * convergence loop per field (src/cuda/geodesics_ptp.cu:206-229).
 *
 * Parameters: a flat float array of gp_mlp_n_params() values,
 * W1[GP_MLP_IN][64] b1[64] W2[64][64] b2[64] W3[64][2] b3[2].
 * All arrays below are host arrays.
 */
#define GP_MLP_IN 16
uint32_t gp_mlp_n_params(void);
/* One forward/backward pass of the mean squared error over n samples:
 * X[n][GP_MLP_IN], T[n][2] -> grads[n_params], *loss. */
gp_status gp_mlp_grad(gp_ctx *ctx, const float *X, const float *T, uint32_t n, const float *params,
                      float *grads, float *loss);
/* Full-batch Adam for `epochs` steps at learning rate lr; params updated in
 * place; losses[epochs] (may be null) receives the loss before each step. */
gp_status gp_mlp_train(gp_ctx *ctx, const float *X, const float *T, uint32_t n, float *params, uint32_t epochs,
                       float lr, float *losses);
/* Y[n][2] = MLP(X): bf16 != 0 uses the BF16 tensor-core kernel (FP32
 * accumulation), else the FP32 kernels of training. */
gp_status gp_mlp_infer(gp_ctx *ctx, const float *X, uint32_t n, const float *params, float *Y, int bf16);

/*
 * Autotuner: time the batch `fields` (as gp_ptp_batch would run it, `reps`
 * times per candidate, best device time) over the one-CTA window widths
 * 1024..16384 with the lockstep grid launch, then the work-queue launch with
 * tiles of 64, 128 and 256 vertices at the best width, and write the fastest
 * setting into opts->local_window / grid_kernel / queue_tile (the other
 * members are kept).  The fields' outputs are written by every candidate run;
 * all candidates give identical results.  No reference counterpart (gproshan
 * uses fixed NT/NB launch constants, include/cuda/geodesics_ptp.cuh:7-8).
 */
gp_status gp_ptp_autotune(gp_ctx *ctx, const gp_field *fields, uint32_t n_fields, gp_dtype dist_type,
                          uint32_t flags, gp_ptp_opts *opts, uint32_t reps);

/*
 * Plans: one batched call captured once in a CUDA graph and replayed.
 * The fields' sources and dist are DEVICE pointers (as with
 * GP_BATCH_DEVICE_POINTERS) that stay valid for the plan's life: write new
 * source ids (same counts) into them between launches.  clusters must be
 * null; at most 2048 fields.  The plan owns its device workspace and a copy
 * of the context's cost model taken at creation.  gp_plan_launch enqueues the
 * graph on `stream` (null: the context's stream) and returns; gp_plan_wait
 * synchronises `stream`, reports device-side errors and fills per-field stats
 * (may be null; seconds is 0).  One launch of a plan at a time.  No reference
 * counterpart (the reference runs every call step by step from the host).
 */
typedef struct gp_plan gp_plan;
gp_status gp_plan_create(gp_ctx *ctx, const gp_field *fields, uint32_t n_fields, const gp_ptp_opts *opts,
                         gp_dtype dist_type, gp_plan **plan);
gp_status gp_plan_launch(gp_plan *plan, void *stream);
gp_status gp_plan_wait(gp_plan *plan, void *stream, gp_ptp_stats *stats);
void gp_plan_destroy(gp_plan *plan);

/* Install (params != null, gp_mlp_n_params() floats) or remove the cost model
 * used by GP_SCHED_LEARNED on this context. */
gp_status gp_ctx_set_cost_model(gp_ctx *ctx, const float *params);
/* The GP_MLP_IN features of each field (toplesets computed on the GPU, no
 * sweep): features[n_fields][GP_MLP_IN], host array.  The fields' dist,
 * clusters and stats members are not used. */
gp_status gp_field_features(gp_ctx *ctx, const gp_field *fields, uint32_t n_fields, float *features);

/*
 * OFF input (che_off::read_file, src/che_off.cpp:28-79): OFF, COFF and NOFF
 * files, triangles and quads (a quad a b c d becomes (a, b, c) and (d, a, c)
 * as in the reference), '#' comments skipped.  The counts are always
 * written; xyz (3 doubles per vertex) and VT (3 indices per triangle) are
 * filled when not null and large enough (else GP_ERR_CAPACITY), so a first
 * call with null arrays gives the sizes.  Host only, no device needed.
 */
gp_status gp_off_read(const char *path, uint32_t *n_vertices, uint32_t *n_faces, double *xyz, uint32_t cap_vertices,
                      uint32_t *VT, uint32_t cap_faces);
/* An OFF file straight to a device mesh: read, upload, half-edge tables
 * built on the GPU (che::init(file), src/che.cpp:1266-1273). */
gp_status gp_mesh_create_off(gp_ctx *ctx, const char *path, gp_mesh **mesh);
/* The half-edge tables of gp_che_build computed on the GPU (host arrays in
 * and out; the same OT, EVT and manifold flag, non-manifold rules included).
 * GP_ERR_CAPACITY if an edge is shared by more than 32 half-edges or a vertex
 * has more than 32 border half-edges (gp_mesh_create then builds on the
 * host).  gp_mesh_create uses this build whenever OT/EVT are not given. */
gp_status gp_che_build_device(gp_ctx *ctx, uint32_t n_vertices, uint32_t n_faces, const uint32_t *VT, uint32_t *OT,
                              uint32_t *EVT, int *manifold);

/*
 * Test hook for the bounded waits (no reference counterpart).  spin_limit:
 * polls before the lockstep grid barrier gives up (0: the built-in limit,
 * about a second or more); phantom_arrivals: arrivals the barrier waits for
 * beyond the CTAs launched, so that with a value > 0 the wait cannot end and
 * the call must report GP_ERR_DEVICE_TIMEOUT after spin_limit polls, with the
 * context still usable.  Leave both 0 in normal use.
 */
gp_status gp_ctx_debug_barrier(gp_ctx *ctx, uint32_t spin_limit, uint32_t phantom_arrivals);

/* normalize_ptp (src/geodesics_ptp.cpp:264-276) on a host array. */
gp_status gp_normalize_ptp(gp_ctx *ctx, void *dist, gp_dtype dist_type, uint64_t n);

/*
 * Farthest-point sampling by repeated multi-source PTP
 * (farthest_point_sampling_ptp_gpu, src/cuda/geodesics_ptp.cu:87-172).
 * samples: host array of capacity cap holding n_init seeds on entry.
 * n: requested number of samples (clamped to n_vertices/2 as the reference
 * does); stops early once the farthest distance drops to radio or below.
 * *n_out receives the number of samples, *max_dist the last farthest distance.
 */
gp_status gp_fps(gp_ctx *ctx, gp_mesh *mesh, uint32_t *samples, uint32_t n_init, uint32_t cap,
                 uint64_t n, double radio, const gp_ptp_opts *opts, uint32_t *n_out,
                 double *max_dist, double *seconds);

#ifdef __cplusplus
}
#endif

#endif /* GP_PTP_H */
