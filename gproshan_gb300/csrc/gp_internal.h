// Internal types shared by the host glue (gp_capi.cpp) and the CUDA kernels.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>
#include <string>
#include <vector>

#include "../../include/gp_ptp.h"

namespace gp {

constexpr uint32_t NIL = 0xFFFFFFFFu;
constexpr uint32_t FAN_CLOSED = 0x80000000u;  // bit 31 of fan_off[v]: v's fan is closed
constexpr uint32_t FAN_MASK = 0x7FFFFFFFu;
constexpr uint32_t MAX_WALK = 1u << 16;       // longest star walk accepted per vertex
// Fixed-stride fan rows: slots 0..n-1 hold the fan; bit 31 of slot 0 marks a
// closed fan; a vertex with more than 8 fan entries has slot 7 = FAN8_OVERFLOW
// and is read from the CSR lists (off/fan) instead.  The mesh's own rows mark
// unused slots FAN8_EMPTY.  The renumbered rows of a field pad them instead: a
// closed fan repeats its first neighbour in slot n, the remaining slots repeat
// the last entry written, and a closed fan of 8 entries overflows.
constexpr uint32_t FAN8_EMPTY = 0xFFFFFFFFu;
constexpr uint32_t FAN8_OVERFLOW = 0xFFFFFFFEu;
// Slot 0 of a renumbered field row (the FP32 sweeps' rows) also carries the
// row's entry count: bit 31 closed, bits 27-30 count (0-8), bits 0-26 the
// first neighbour (a field's renumbered ids stay below 2^27, checked on the host).
constexpr uint32_t FAN8_N_SHIFT = 27;
constexpr uint32_t FAN8_ID_MASK = (1u << FAN8_N_SHIFT) - 1u;
constexpr uint64_t FIELD_MAX_SLOTS_F32 = 1ull << FAN8_N_SHIFT;

// trig/next/prev of the compact half-edge mesh (src/che.cpp:18-34)
__host__ __device__ inline uint32_t he_next(uint32_t he) { return 3 * (he / 3) + (he + 1) % 3; }
__host__ __device__ inline uint32_t he_prev(uint32_t he) { return 3 * (he / 3) + (he + 2) % 3; }

// device error bits (GridSync::err)
constexpr uint32_t DEV_ERR_TIMEOUT = 1u;   // a grid-barrier wait ran past its limit
constexpr uint32_t DEV_ERR_WALK = 2u;      // a star walk did not close
constexpr uint32_t DEV_ERR_BOUNDS = 4u;    // an index outside its buffer

// Barrier / abort word of one persistent launch.
struct GridSync {
	uint32_t count;  // CTAs arrived at the current barrier
	uint32_t gen;    // barrier generation
	uint32_t err;    // DEV_ERR_* bits
	uint32_t abort;  // set once any CTA gives up; the others leave at their next barrier
};

// Work-queue sweeps (ptp_queue_kernel).  Each queued field has QUEUE_STRIPES
// claim cursors (one 128-byte line each, so claims on different stripes hit
// different L2 lines) and as many completion counters.  A cursor packs
// epoch (12 bits, the field's sweep number mod 4096) | tiles (26) | next tile (26).
constexpr uint32_t QUEUE_STRIPES = 4;
// words of the lockstep grid launch's barrier block: [0] top arrivals, [1]
// abort, [2] error bits, [3] steps, then 16 group counters on 128-byte lines
constexpr uint32_t GRID_BAR_WORDS = 32;  // one 128-byte line: see count_barrier
// the barrier words of the launch that resumes after a streaming launch: the
// line's second half (errors, steps and skip counts are read from both)
constexpr uint32_t BAR_RESUME = GRID_BAR_WORDS / 2;
constexpr uint32_t GRID_NONE = 0, GRID_LOCKSTEP = 1, GRID_QUEUE = 2;
// Streamed fields (gp_ptp.cu, stream_worker): toplesets and renumbering built
// by worker CTAs of the lockstep launch while the other CTAs sweep.
constexpr uint32_t STREAM_MAX = 32;         // streamed fields per launch
constexpr uint32_t STREAM_PER_WORKER = 2;   // fields one worker CTA interleaves (1: same speed, twice the workers)
constexpr uint32_t STREAM_MARGIN = 16;      // slots past a window's reads that must be final
constexpr uint32_t STREAM_ALIGN = 32;       // field bases (slots) with streamed fields: 128 bytes of 32-bit entries

struct alignas(128) QLine {
	unsigned long long w;
	uint32_t pad[30];
};

// Schedule of one queued field; only the warp that completes a sweep reads
// and writes it (relaxed loads and stores, ordered by the completion counters).
struct QField {
	uint4 sched[2];      // per epoch parity: win_s, win_e, chk_e, d | groups << 1
	uint32_t f;          // field id
	uint32_t n_limits, max_iter, i, j, d, iter, n_iter;
	uint32_t notok[2];   // per epoch parity: a ring-i vertex failed the test
	uint32_t pad[2];
	unsigned long long relax;
};

struct QCtl {
	uint32_t G;          // fields handed to the grid-wide sweeps
	uint32_t mode;       // GRID_NONE, GRID_LOCKSTEP or GRID_QUEUE
	uint32_t live;       // queued fields still running
	uint32_t progress;   // sweeps completed by the queue kernel
	uint32_t abort;
	uint32_t err;        // DEV_ERR_* bits
	uint32_t warps;      // warps of the queue launch
	uint32_t groups;     // 32-vertex groups per claimed tile; 0: chosen per window
};

// A mesh on the device, original vertex numbering.
struct MeshDev {
	const float4 *pos;       // nv (x, y, z, 0)
	const double *posd;      // 4*nv (x, y, z, 0); null unless the FP64 path is enabled
	const uint32_t *fan_off; // nv+1; entries [fan_off[v]&MASK, fan_off[v+1]&MASK); bit31 = closed
	const uint32_t *fan;     // link of each vertex in star-walk order (che::link order)
	const uint4 *fan8;       // 2 * nv: the same links as fixed-stride rows (FAN8_* encoding)
	uint32_t nv;
	uint32_t n_fan;
	uint32_t max_fan;        // largest per-vertex entry count
	uint32_t pad;
	// geometry statistics (cost-model features): log mean edge, edge-length
	// coefficient of variation, std of log edge length, obtuse-triangle
	// fraction, mean (1 - cos) of dihedral angles
	float stats[5];
	float pad2[3];
};

// Buffers of one field (one source set on one mesh) on the device.
struct FieldDev {
	MeshDev m;
	const uint32_t *src;      // ns sources
	uint32_t ns;
	uint32_t cap_sorted;      // nv + ns
	// toplesets
	uint32_t *ring;           // nv
	unsigned long long *key;  // nv: BFS discovery key (frontier position << 20 | link slot)
	uint32_t *sorted;         // cap_sorted
	uint32_t *limits;         // nv + 2
	// ring-renumbered copy: new id k = position k of sorted; id nr = "unreached" sentinel
	uint32_t *inv;            // nv: old -> new id (sentinel if unreached)
	float4 *P;                // cap_sorted + 1
	double *Pd;               // 4*(cap_sorted + 1) or null
	uint32_t *off;            // cap_sorted + 2 (bit31 = closed)
	uint32_t *fan;            // renumbered fan entries
	uint4 *fan8;              // 2 * (cap_sorted + 1): 8 fan slots per vertex (see FAN8_*)
	void *D[2];               // cap_sorted + 1 distances (float or double)
	uint32_t *C[2];           // cap_sorted + 1 labels, or null
	// outputs / inputs in original numbering
	void *dist_out;           // nv of out_dtype
	uint32_t *clusters_out;   // nv or null
	const uint32_t *clusters_in; // nv initial labels or null
	uint32_t *trace;          // 2 * trace_cap (i, j) per sweep or null
	uint32_t trace_cap;
	uint32_t out_f64;         // 1: dist_out is double
	uint32_t max_iter;        // 0: 2 * n_limits
	uint32_t round_coords;    // FP64 path on the float-rounded coordinates
	double tol;
	float tol32;              // tol rounded to float (the FP32 path's ring test)
	uint32_t stream;          // 1: toplesets and renumbering run inside the lockstep launch (stream_*)
};

// Device-side state of a farthest-point sampling loop (gp_fps).
struct FpsDev {
	uint32_t ns;                // samples so far (the field's source count)
	uint32_t ns_max;            // capacity of the sample array
	uint32_t stop;              // the loop has ended (radius reached, array full, or a device error)
	uint32_t err;               // DEV_ERR_* bits seen by any sample
	double max_dist;            // max |d| of the last sample's field
	unsigned long long amax;    // max |d| bits of the current field (gather), reset by the append
	uint32_t first;             // first vertex holding amax (fps_first_kernel), reset by the append
	uint32_t pad2;
};

// Mutable per-field state of the persistent launches.
struct FieldState {
	// toplesets
	uint32_t n_limits;   // |limits| once the BFS is finished
	uint32_t bfs_live;   // 1 while the BFS of this field runs
	uint32_t status;     // DEV_ERR_* of this field
	// PTP schedule (run_ptp_gpu, src/cuda/geodesics_ptp.cu:198-229)
	uint32_t i, j, d, iter, max_iter, n_iter, live;
	uint32_t win_s, win_e, chk_e, nr;  // current window, check-ring end, reached vertices
	uint32_t big;        // 1: swept by the grid-wide launch, 0: by one CTA
	unsigned long long relax;
	unsigned long long nmax;  // largest finite positive output (bits), for gp_ptp_opts::normalize
};


// Where a sample's device errors are (all cleared before each sample runs).
struct FpsErr {
	const GridSync *sync;       // 2: BFS / sweep barrier words
	const uint32_t *bar;        // lockstep barrier block ([2] = error bits)
	const QCtl *ctl;            // work-queue control
	const FieldState *state;    // the field's state (status)
	const uint32_t *wbar;       // whole-GPU BFS barrier block, or null
};

// ------------------------------------------------------------------
// Kernel entry points implemented in the .cu files (all asynchronous on `s`).
// ------------------------------------------------------------------

// gp_mesh.cu
cudaError_t launch_fan_count(const uint32_t *VT, const uint32_t *OT, const uint32_t *EVT, uint32_t nv,
                             uint32_t nhe, uint32_t *cnt, uint32_t *err, cudaStream_t s);
cudaError_t launch_pos_convert(const double *xyz, uint32_t nv, float4 *pos, double *posd, cudaStream_t s);

// exclusive scan of n u32 values (in place allowed); out[n] receives the total.
// tmp needs scan_tmp_words(n) words.
size_t scan_tmp_words(size_t n);
cudaError_t launch_scan_u32(const uint32_t *in, uint32_t *out, size_t n, uint32_t *tmp, cudaStream_t s);
cudaError_t launch_max_u32(const uint32_t *in, size_t n, uint32_t *out, cudaStream_t s);

// gp_toplesets.cu: BFS of all fields (taken in `order`, or by index if null);
// fills ring/sorted/limits and state[f].n_limits.
cudaError_t launch_toplesets(FieldDev *fields, FieldState *state, uint32_t n_fields, uint32_t *queue,
                             uint32_t ctas, const uint32_t *order, cudaStream_t s);
int toplesets_max_ctas(int device);
size_t che_build_scratch_bytes(uint32_t nv, uint32_t nhe);
gp_status off_parse(const char *path, std::vector<double> &xyz, std::vector<uint32_t> &tri, std::string &err);
cudaError_t launch_che_build(const uint32_t *VT, uint32_t nv, uint32_t nhe, uint32_t *OT, uint32_t *EVT,
                             void *scratch, uint32_t *flags, cudaStream_t s);
int toplesets_wide_ctas(int device);
cudaError_t launch_toplesets_wide(FieldDev *fields, FieldState *state, const uint32_t *wide, uint32_t n_wide,
                                  uint32_t *bar, uint32_t *cta_tot, uint32_t ctas, cudaStream_t s);

// gp_ptp.cu
int ptp_max_ctas(int device, bool f64, bool clusters, uint32_t n_fields);

// gp_mesh.cu: sums for the geometry statistics (8 doubles, zeroed by the caller):
// [0] sum l, [1] sum l^2, [2] sum log l, [3] sum (log l)^2, [4] edges,
// [5] obtuse faces, [6] sum (1 - cos dihedral), [7] interior edges
cudaError_t launch_mesh_stats(const uint32_t *VT, const uint32_t *OT, const float4 *pos, uint32_t nf, double *acc,
                              cudaStream_t s);

// gp_capi.cpp: a mesh's device arrays and the device that holds them
const MeshDev *mesh_dev(const gp_mesh *mesh);
int mesh_device(const gp_mesh *mesh);

} // namespace gp
