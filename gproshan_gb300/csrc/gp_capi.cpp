// C ABI of libgp_ptp.so (include/gp_ptp.h): argument checks, device workspace,
// per-call layout of the field buffers, and the launch sequence
//   toplesets (BFS) -> ring renumbering -> persistent sweeps -> gather.
#include <algorithm>
#include <cmath>
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cstdarg>
#include <mutex>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gp_internal.h"
#include "gp_mlp.h"

namespace gp {
// launchers defined in the .cu files and not in gp_internal.h's first list
cudaError_t launch_fan_fill(const uint32_t *VT, const uint32_t *OT, const uint32_t *EVT, uint32_t nv,
                            const uint32_t *flags, uint32_t *off, uint32_t *fan, cudaStream_t s);
cudaError_t launch_strip_flags(const uint32_t *in, uint32_t *out, uint32_t n, cudaStream_t s);
cudaError_t launch_fan8(const uint32_t *off, const uint32_t *fan, uint32_t nv, uint4 *rows, cudaStream_t s);
cudaError_t launch_bfs_setup(FieldDev *fields, FieldState *state, const uint32_t *vbase, uint32_t n_fields,
                             uint32_t total_vertices, cudaStream_t s);
cudaError_t launch_renumber_batch(FieldDev *fields, FieldState *state, const uint32_t *base, uint32_t n_fields,
                                  uint32_t total, uint32_t *cnt, uint32_t *scan_tmp, bool f64, bool clusters,
                                  bool csr, bool inv_ready, cudaStream_t s);
cudaError_t launch_gather_batch(FieldDev *fields, FieldState *state, const uint32_t *base, uint32_t n_fields,
                                uint32_t total, bool f64, bool clusters, cudaStream_t s, unsigned long long *amax = nullptr, bool nmax = false);
cudaError_t launch_normalize_batch(FieldDev *fields, FieldState *state, const uint32_t *base, uint32_t n_fields,
                                   uint32_t total, bool out_f64, cudaStream_t s);
cudaError_t launch_normalize(void *dist, bool f64, uint64_t n, unsigned long long *tmp, cudaStream_t s);
cudaError_t launch_fps_sources(FieldDev *field, const FpsDev *c, cudaStream_t s);
cudaError_t launch_fps_append(const void *dist, bool f64, uint32_t n, FpsDev *c, uint32_t *samples, double radio,
                              const FpsErr &e, cudaStream_t s);
int ptp_local_max_ctas(int device, bool f64, bool clusters);
cudaError_t launch_classify(FieldDev *fields, FieldState *state, uint32_t n_fields, uint32_t local_window,
                            const uint32_t *pred_big, cudaStream_t s);
cudaError_t launch_ptp_local(FieldDev *fields, FieldState *state, uint32_t n_fields, uint32_t *queue,
                             uint32_t ctas, uint32_t local_window, const uint32_t *perm, bool f64, bool clusters,
                             cudaStream_t s);
cudaError_t launch_field_features(const FieldDev *fields, const FieldState *state, uint32_t n_fields, float *out,
                                  cudaStream_t s);
cudaError_t launch_plan(const FieldDev *fields, const FieldState *state, uint32_t n_fields, const float *pred,
                        uint32_t local_window, uint32_t *pred_big, float *cost, uint32_t *perm, cudaStream_t s);
cudaError_t launch_ptp(FieldDev *fields, FieldState *state, uint32_t n_fields, uint32_t *notok, uint32_t *bar,
                       uint32_t ctas, bool f64, bool clusters, unsigned long long *steps, uint32_t steps_cap,
                       const QCtl *ctl, uint32_t spin_limit, uint32_t phantom, const uint32_t *sids,
                       uint32_t n_stream, uint32_t workers, unsigned long long *sprog, unsigned long long *snap,
                       cudaStream_t s);
cudaError_t launch_ptp_queue(FieldDev *fields, FieldState *state, uint32_t n_fields, QField *qf, QLine *cur,
                             QLine *done, QLine *sdone, QCtl *ctl, uint32_t ctas, uint32_t mode_req,
                             uint32_t min_queue, uint32_t tile, bool f64, bool clusters, cudaStream_t s);
int ptp_queue_max_ctas(int device, bool f64, bool clusters);
uint32_t ptp_grid_max_fields();
size_t ptp_snap_words(uint32_t n_fields);
int ptp_binary_version();
} // namespace gp

using namespace gp;

struct gp_ctx {
	int device = 0;
	cudaStream_t stream = nullptr;
	int num_sms = 0;
	std::string err;
	void *ws = nullptr;        // grow-only device workspace
	size_t ws_bytes = 0;
	void *pin = nullptr;       // grow-only pinned host staging
	size_t pin_bytes = 0;
	cudaEvent_t ev0 = nullptr, ev1 = nullptr;
	cudaEvent_t ph[6] = {};    // phase boundaries of the last call
	cudaEvent_t fps0 = nullptr, fps1 = nullptr;  // start / end of a farthest-point sampling loop
	gp_call_stats last{};
	unsigned long long *steps = nullptr;   // grid-launch step trace (device), if enabled
	uint32_t steps_cap = 0;
	int bfs_ctas = 0;
	int bfs_wide_ctas = 0;     // CTAs of the wide-field BFS launch (all resident)
	int ptp_ctas[4] = {0, 0, 0, 0};
	int local_ctas[4] = {0, 0, 0, 0};
	uint32_t grid_ctas = 0;    // CTAs of the last grid launch
	int queue_ctas[4] = {};    // CTAs of the work-queue launch (all resident) per variant
	float *model = nullptr;    // cost-model parameters (device), or null
	uint32_t dbg_spin = 0;     // grid-barrier poll limit (0: the default)
	uint32_t dbg_phantom = 0;  // extra arrivals the grid barrier waits for (tests of the bounded wait)
	unsigned long long cu_id = 0;  // id of the CUDA context the handles above belong to (0: unknown)
};

struct gp_mesh {
	gp_ctx *ctx = nullptr;
	int device = 0;
	unsigned long long cu_id = 0;  // CUDA context the block was allocated in (0: unknown)
	uint32_t nv = 0, nf = 0;
	MeshDev dev{};
	void *block = nullptr;     // one device allocation holding the mesh arrays
};

// One batched call captured in a CUDA graph, with its own workspace.
struct gp_plan {
	gp_ctx *ctx = nullptr;
	void *ws = nullptr;
	cudaGraph_t graph = nullptr;
	cudaGraphExec_t exec = nullptr;
	uint32_t n_fields = 0;
	FieldState *state = nullptr;  // device, per field
	QCtl *ctl = nullptr;
	uint32_t *bar = nullptr;
	GridSync *sync = nullptr;
};

namespace {

// kernels launched by launch_scan_u32 for n elements
uint32_t scan_launches(size_t n)
{
	const size_t tile = 1024;
	return n <= tile ? 1u : 2u + scan_launches((n + tile - 1) / tile);
}

void set_err(gp_ctx *ctx, const char *fmt, ...)
{
	if(!ctx) return;
	char buf[512];
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(buf, sizeof(buf), fmt, ap);
	va_end(ap);
	ctx->err = buf;
}

#define GP_CUDA(ctx, call)                                                                     \
	do {                                                                                       \
		cudaError_t e_ = (call);                                                               \
		if(e_ != cudaSuccess)                                                                  \
		{                                                                                      \
			set_err(ctx, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
			return e_ == cudaErrorMemoryAllocation ? GP_ERR_OUT_OF_MEMORY : GP_ERR_CUDA;        \
		}                                                                                      \
	} while(0)

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Offsets of the buffers of one call inside the workspace.
struct Carve {
	size_t off = 0;
	template <class T> size_t add(size_t n)
	{
		off = align_up(off, 256);
		const size_t o = off;
		off += std::max<size_t>(n, 1) * sizeof(T);
		return o;
	}
};

gp_status ensure_ws(gp_ctx *ctx, size_t bytes)
{
	if(bytes <= ctx->ws_bytes) return GP_OK;
	if(ctx->ws)
	{
		GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
		GP_CUDA(ctx, cudaFree(ctx->ws));
		ctx->ws = nullptr;
		ctx->ws_bytes = 0;
	}
	const size_t want = align_up(bytes + bytes / 8, 1 << 20);
	GP_CUDA(ctx, cudaMalloc(&ctx->ws, want));
	ctx->ws_bytes = want;
	return GP_OK;
}

gp_status ensure_pin(gp_ctx *ctx, size_t bytes)
{
	if(bytes <= ctx->pin_bytes) return GP_OK;
	if(ctx->pin)
	{
		GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
		GP_CUDA(ctx, cudaFreeHost(ctx->pin));
		ctx->pin = nullptr;
		ctx->pin_bytes = 0;
	}
	const size_t want = align_up(bytes + bytes / 8, 1 << 16);
	GP_CUDA(ctx, cudaMallocHost(&ctx->pin, want));
	ctx->pin_bytes = want;
	return GP_OK;
}

bool is_device_ptr(const void *p)
{
	cudaPointerAttributes a;
	if(cudaPointerGetAttributes(&a, p) != cudaSuccess)
	{
		cudaGetLastError();
		return false;
	}
	return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// One field request of a call.
struct Req {
	gp_mesh *mesh;
	const uint32_t *src;
	uint32_t ns;
	const uint32_t *limits;   // host toplesets or null
	uint32_t nl;
	const uint32_t *sorted;
	void *dist;               // output (host or device)
	uint32_t *clusters;       // in/out labels or null
	gp_ptp_stats *stats;
};

enum class Stage { toplesets, features, ptp };

// GP_GRID_AUTO takes the work queue from this many grid fields on
constexpr uint32_t QUEUE_MIN_DEFAULT = 0xFFFFFFFFu;
// Default window above which a field leaves the one-CTA launch, per precision.
constexpr uint32_t LOCAL_WINDOW_F32 = 4096u, LOCAL_WINDOW_F64 = 256u;

// Toplesets of a call with at most WIDE_MAX_FIELDS fields run every field on
// a mesh of at least WIDE_MIN_VERTICES vertices on the whole GPU (one level
// at a time, all CTAs); the others one CTA per field.
constexpr uint32_t WIDE_MAX_FIELDS = 8;
constexpr uint32_t WIDE_MIN_VERTICES = 1u << 18;
// Streamed fields (FP32 distances, lockstep grid launch; gp_ptp_opts::stream_min):
// fields on meshes of at least stream_min vertices build their toplesets inside
// the sweep launch.  By default (stream_min 0) STREAM_DEFAULT_MIN, but only in
// calls whose large fields would otherwise build their toplesets on one CTA
// each (more than WIDE_MAX_FIELDS fields, or no whole-GPU BFS): there the
// streamed launch hides the toplesets (benchmark batch 89.7 -> 86.8 ms); a call
// of a few large fields is faster with the whole-GPU BFS first (2048^2 grid,
// one field: 65 ms, streamed 86 ms).
constexpr uint32_t STREAM_NEVER = 0xFFFFFFFFu;
constexpr uint32_t STREAM_DEFAULT_MIN = 1u << 18;

struct TopOut {  // host outputs of gp_toplesets
	uint32_t *rings;
	uint32_t *sorted;
	uint32_t cap_sorted;
	uint32_t *limits;
	uint32_t cap_limits;
	uint32_t *n_limits;
};

// A farthest-point sampling loop run by one call of run(): up to n_iter
// samples appended to the device copy of samples[0, n_init), with no host
// round trip per sample (see fps_append_kernel).
struct FpsLoop {
	uint32_t *samples;    // host: n_init seeds in, the appended samples out (capacity n_init + n_iter)
	uint32_t n_init;
	uint32_t n_iter;      // samples to take at most
	double radio;         // stop once the farthest distance is <= radio
	uint32_t n_out;       // out: samples in total
	double max_dist;      // out: farthest distance of the last sample's field
};

gp_status map_dev_err(gp_ctx *ctx, uint32_t err, const char *where)
{
	if(!err) return GP_OK;
	if(err & DEV_ERR_TIMEOUT)
	{
		set_err(ctx, "%s: a device-side barrier wait ran past its limit", where);
		return GP_ERR_DEVICE_TIMEOUT;
	}
	set_err(ctx, "%s: device reported an index outside its buffer (err=%u)", where, err);
	return GP_ERR_INVALID_ARG;
}

gp_status run(gp_ctx *ctx, const Req *reqs, uint32_t F, const gp_ptp_opts *opts, gp_dtype out_type,
              bool src_dev, bool out_dev, Stage stage, const TopOut *top, double *seconds, float *features = nullptr,
              gp_plan *plan = nullptr, FpsLoop *fps = nullptr)
{
	if(fps && (F != 1 || stage != Stage::ptp || plan || src_dev || out_dev || reqs[0].clusters)) return GP_ERR_INVALID_ARG;
	if(!ctx) return GP_ERR_INVALID_ARG;
	if(!F) return GP_OK;
	const gp_ptp_opts o = opts ? *opts : gp_ptp_opts{};
	const bool f64 = o.precision == GP_F64;
	const bool clusters = stage == Stage::ptp && std::any_of(reqs, reqs + F, [](const Req &r) { return r.clusters; });
	const bool given_tops = reqs[0].limits != nullptr;
	const size_t tsz = 8;  // double (FP64 path) or a (hi, lo) float pair (FP32 path)
	const size_t osz = out_type == GP_F64 ? sizeof(double) : sizeof(float);

	// ---- streamed fields ------------------------------------------------------
	// Streamed fields: the largest FP32 fields whose rows fit the padded fan
	// rows, when the grid launch is the lockstep one (see stream_worker).
	std::vector<uint32_t> sids;
	const bool wide_bfs = F <= WIDE_MAX_FIELDS && ctx->bfs_wide_ctas > 0;
	const uint32_t smin = o.stream_min ? o.stream_min : wide_bfs ? STREAM_NEVER : STREAM_DEFAULT_MIN;
	const bool lockstep = o.grid_kernel == GP_GRID_LOCKSTEP || (o.grid_kernel == GP_GRID_AUTO && !o.queue_min);
	if(stage == Stage::ptp && !f64 && !clusters && !fps && !given_tops && lockstep && smin != STREAM_NEVER)
	{
		for(uint32_t f = 0; f < F; f++)
			if(reqs[f].mesh && reqs[f].mesh->nv >= smin && reqs[f].mesh->dev.max_fan <= 7) sids.push_back(f);
		std::stable_sort(sids.begin(), sids.end(),
		                 [&](uint32_t x, uint32_t y) { return reqs[x].mesh->nv > reqs[y].mesh->nv; });
		if(sids.size() > STREAM_MAX) sids.resize(STREAM_MAX);
	}
	const int maxc = stage == Stage::ptp ? ptp_max_ctas(ctx->device, f64, clusters, F) : 0;
	const uint32_t ctas = o.ctas ? std::min<uint32_t>(o.ctas, (uint32_t) maxc) : (uint32_t) maxc;
	// Workers: the fields of at least 3/4 of the largest's vertices (the
	// longest BFS) get a worker each, the others two per worker, the largest
	// of them with the smallest.  Worker w builds the fields at positions w and
	// w + workers (gp_ptp.cu: stream_worker), so the order is: the larger
	// halves of the pairs, the solo fields, the smaller halves reversed.
	// (Benchmark batch, grid phase: pairs by size order 80.4 ms, largest with
	// smallest 79.9; the same box, pairs only 79.78 against the 1M-vertex
	// fields solo 79.62.)  Workers take at most a quarter of the launch's CTAs.
	static_assert(STREAM_PER_WORKER == 2, "the order below pairs fields two per worker");
	uint32_t workers = 0;
	for(;;)
	{
		const uint32_t n = (uint32_t) sids.size();
		uint32_t solo = 0;
		while(solo < n && 4ull * reqs[sids[solo]].mesh->nv >= 3ull * reqs[sids[0]].mesh->nv) solo++;
		workers = solo + (n - solo + STREAM_PER_WORKER - 1) / STREAM_PER_WORKER;
		if(workers <= ctas / 4 || sids.empty()) break;
		sids.pop_back();
	}
	const uint32_t n_stream = (uint32_t) sids.size();
	if(n_stream)
	{
		uint32_t solo = 0;
		while(solo < n_stream && 4ull * reqs[sids[solo]].mesh->nv >= 3ull * reqs[sids[0]].mesh->nv) solo++;
		const uint32_t rest = n_stream - solo, big = (rest + 1) / 2;
		std::vector<uint32_t> o;
		o.insert(o.end(), sids.begin() + solo, sids.begin() + solo + big);  // positions [0, big)
		o.insert(o.end(), sids.begin(), sids.begin() + solo);                // [big, workers)
		for(uint32_t k = n_stream; k-- > solo + big;) o.push_back(sids[k]);   // [workers, n)
		sids.swap(o);
	}

	// ---- checks and layout -------------------------------------------------
	std::vector<uint32_t> base(F + 1), vbase(F + 1), fbase(F + 1), sbase(F + 1);
	uint64_t tot = 0, vtot = 0, ftot = 0, stot = 0;
	for(uint32_t f = 0; f < F; f++)
	{
		const Req &r = reqs[f];
		if(!r.mesh || r.mesh->ctx != ctx || !r.src || !r.ns)
		{
			set_err(ctx, "field %u: null mesh/sources, empty source list, or mesh of another context", f);
			return GP_ERR_INVALID_ARG;
		}
		if(stage == Stage::ptp && !r.dist)
		{
			set_err(ctx, "field %u: null dist", f);
			return GP_ERR_INVALID_ARG;
		}
		if(given_tops != (r.limits != nullptr) || (r.limits && (!r.sorted || r.nl < 1 || F != 1)))
		{
			set_err(ctx, "toplesets must be given for a single field with both limits and sorted");
			return GP_ERR_INVALID_ARG;
		}
		const uint32_t nv = r.mesh->nv;
		if(!src_dev)
			for(uint32_t s = 0; s < (fps ? fps->n_init : r.ns); s++)
				if(r.src[s] >= nv)
				{
					set_err(ctx, "field %u: source %u = %u out of range (n_vertices %u)", f, s, r.src[s], nv);
					return GP_ERR_INVALID_ARG;
				}
		// no 128-byte line of a renumbered array or of the limits spans two fields
		if(n_stream) tot = align_up(tot, STREAM_ALIGN);
		base[f] = (uint32_t) tot;
		vbase[f] = (uint32_t) vtot;
		fbase[f] = (uint32_t) ftot;
		sbase[f] = (uint32_t) stot;
		const uint64_t S = (uint64_t) nv + r.ns + 2;
		if(stage == Stage::ptp && !f64 && S >= FIELD_MAX_SLOTS_F32)
		{
			set_err(ctx, "field %u: %llu vertices and sources exceed the FP32 path's 2^27 per field (use GP_F64)", f,
			        (unsigned long long) S);
			return GP_ERR_CAPACITY;
		}
		tot += S;
		vtot += nv;
		ftot += (uint64_t) r.mesh->dev.n_fan + (uint64_t) r.ns * r.mesh->dev.max_fan;
		stot += r.ns;
	}
	base[F] = (uint32_t) tot;
	vbase[F] = (uint32_t) vtot;
	fbase[F] = (uint32_t) ftot;
	sbase[F] = (uint32_t) stot;
	if(tot >= (1ull << 31) || ftot >= (1ull << 31))
	{
		set_err(ctx, "batch too large (%llu slots, %llu fan entries): split it", (unsigned long long) tot,
		        (unsigned long long) ftot);
		return GP_ERR_CAPACITY;
	}
	if(given_tops)
	{
		const Req &r = reqs[0];
		const uint32_t cap = r.mesh->nv + r.ns;
		if(r.nl > r.mesh->nv + 2 || r.limits[r.nl - 1] > cap || r.limits[0] != 0)
		{
			set_err(ctx, "toplesets limits out of range");
			return GP_ERR_INVALID_ARG;
		}
		for(uint32_t k = 1; k < r.nl; k++)
			if(r.limits[k] < r.limits[k - 1])
			{
				set_err(ctx, "toplesets limits not increasing at %u", k);
				return GP_ERR_INVALID_ARG;
			}
		for(uint32_t k = 0; k < r.limits[r.nl - 1]; k++)
			if(r.sorted[k] >= r.mesh->nv)
			{
				set_err(ctx, "toplesets sorted[%u] out of range", k);
				return GP_ERR_INVALID_ARG;
			}
	}

	Carve cv;
	const size_t o_fields = cv.add<FieldDev>(F), o_state = cv.add<FieldState>(F);
	const size_t o_sids = cv.add<uint32_t>(STREAM_MAX), o_sprog = cv.add<unsigned long long>(STREAM_MAX);
	const size_t o_snap = cv.add<unsigned long long>(ptp_snap_words(F));
	const size_t o_sync = cv.add<GridSync>(2), o_base = cv.add<uint32_t>(F + 1), o_vbase = cv.add<uint32_t>(F + 1);
	const size_t o_queue = cv.add<uint32_t>(4);
	const size_t o_notok = cv.add<uint32_t>(3 * (size_t) F), o_bar = cv.add<uint32_t>(GRID_BAR_WORDS);
	const size_t o_feat = cv.add<float>((size_t) F * MLP_IN), o_pred = cv.add<float>((size_t) F * MLP_OUT);
	const size_t o_pbig = cv.add<uint32_t>(F), o_cost = cv.add<float>(F), o_perm = cv.add<uint32_t>(F);
	const size_t o_qf = cv.add<QField>(F), o_qcur = cv.add<QLine>((size_t) F * QUEUE_STRIPES);
	const size_t o_qdone = cv.add<QLine>((size_t) F * QUEUE_STRIPES), o_qsd = cv.add<QLine>(F);
	const size_t o_qctl = cv.add<QCtl>(1), o_model = cv.add<float>(MLP_NPARAM), o_border = cv.add<uint32_t>(F);
	std::vector<uint32_t> wide;
	if(!given_tops && wide_bfs)
		for(uint32_t f = 0; f < F; f++)
			if(reqs[f].mesh->nv >= WIDE_MIN_VERTICES && std::find(sids.begin(), sids.end(), f) == sids.end())
				wide.push_back(f);
	const size_t o_wide = cv.add<uint32_t>(F), o_wbar = cv.add<uint32_t>(4);
	const size_t o_wtot = cv.add<uint32_t>((size_t) std::max(ctx->bfs_wide_ctas, 1));
	const size_t o_ring = cv.add<uint32_t>(tot), o_key = cv.add<unsigned long long>(tot);
	const size_t o_sorted = cv.add<uint32_t>(tot), o_lim = cv.add<uint32_t>(tot), o_inv = cv.add<uint32_t>(tot);
	size_t o_cnt = 0, o_scan = 0, o_P = 0, o_Pd = 0, o_off = 0, o_fan = 0, o_D0 = 0, o_D1 = 0, o_C0 = 0, o_C1 = 0;
	size_t o_fan8 = 0;
	size_t o_out = 0, o_cout = 0, o_cin = 0;
	if(stage == Stage::ptp)
	{
		o_cnt = cv.add<uint32_t>(tot + 1);
		o_scan = cv.add<uint32_t>(scan_tmp_words(tot));
		o_P = cv.add<float4>(tot);
		if(f64) o_Pd = cv.add<double>(4 * tot);
		o_off = cv.add<uint32_t>(tot);
		o_fan8 = cv.add<uint4>(2 * tot);
		o_fan = cv.add<uint32_t>(ftot);
		o_D0 = cv.add<char>(tot * tsz);
		o_D1 = cv.add<char>(tot * tsz);
		if(clusters)
		{
			o_C0 = cv.add<uint32_t>(tot);
			o_C1 = cv.add<uint32_t>(tot);
			o_cout = cv.add<uint32_t>(vtot);
			o_cin = cv.add<uint32_t>(vtot);
		}
		if(!out_dev) o_out = cv.add<char>(vtot * osz);
	}
	const size_t o_src = cv.add<uint32_t>(stot);
	const size_t o_fps = fps ? cv.add<FpsDev>(1) : 0;
	gp_status st = GP_OK;
	if(plan)
	{
		// a plan owns its workspace: later calls on the context cannot move it
		GP_CUDA(ctx, cudaMalloc(&plan->ws, cv.off));
	}
	else
	{
		st = ensure_ws(ctx, cv.off);
		if(st != GP_OK) return st;
	}
	char *W = static_cast<char *>(plan ? plan->ws : ctx->ws);
	auto P = [&](size_t off) { return W + off; };

	// ---- host-side descriptors -------------------------------------------------
	std::vector<FieldDev> hf(F);
	std::vector<FieldState> hs(F);
	std::memset(hs.data(), 0, sizeof(FieldState) * F);
	for(uint32_t f = 0; f < F; f++)
	{
		const Req &r = reqs[f];
		FieldDev &d = hf[f];
		std::memset(&d, 0, sizeof(d));
		d.m = r.mesh->dev;
		d.ns = fps ? fps->n_init : r.ns;  // an FPS field's count grows on the device (capacity r.ns)
		d.cap_sorted = r.mesh->nv + r.ns;
		d.src = src_dev ? r.src : reinterpret_cast<const uint32_t *>(P(o_src)) + sbase[f];
		d.ring = reinterpret_cast<uint32_t *>(P(o_ring)) + base[f];
		d.key = reinterpret_cast<unsigned long long *>(P(o_key)) + base[f];
		d.sorted = reinterpret_cast<uint32_t *>(P(o_sorted)) + base[f];
		d.limits = reinterpret_cast<uint32_t *>(P(o_lim)) + base[f];
		d.inv = reinterpret_cast<uint32_t *>(P(o_inv)) + base[f];
		if(stage == Stage::ptp)
		{
			d.P = reinterpret_cast<float4 *>(P(o_P)) + base[f];
			d.Pd = f64 ? reinterpret_cast<double *>(P(o_Pd)) + 4ull * base[f] : nullptr;
			d.off = reinterpret_cast<uint32_t *>(P(o_off)) + base[f];
			d.fan8 = reinterpret_cast<uint4 *>(P(o_fan8)) + 2ull * base[f];
			d.fan = reinterpret_cast<uint32_t *>(P(o_fan));
			d.D[0] = P(o_D0) + (size_t) base[f] * tsz;
			d.D[1] = P(o_D1) + (size_t) base[f] * tsz;
			if(clusters)
			{
				d.C[0] = reinterpret_cast<uint32_t *>(P(o_C0)) + base[f];
				d.C[1] = reinterpret_cast<uint32_t *>(P(o_C1)) + base[f];
				if(r.clusters)
				{
					d.clusters_out = out_dev ? r.clusters : reinterpret_cast<uint32_t *>(P(o_cout)) + vbase[f];
					d.clusters_in = out_dev ? r.clusters : reinterpret_cast<uint32_t *>(P(o_cin)) + vbase[f];
				}
			}
			d.dist_out = out_dev ? r.dist : P(o_out) + (size_t) vbase[f] * osz;
			d.out_f64 = out_type == GP_F64;
			d.max_iter = o.max_iter;
			d.round_coords = o.round_coords ? 1u : 0u;
			d.tol = o.tol > 0 ? o.tol : GP_PTP_TOL;
			d.tol32 = (float) d.tol;
		}
		if(given_tops) hs[f].n_limits = r.nl;
	}
	for(uint32_t q = 0; q < n_stream; q++) hf[sids[q]].stream = q + 1;
	// in-place label input and output on device pointers would race; stage them
	if(clusters && out_dev)
		for(uint32_t f = 0; f < F; f++)
			if(reqs[f].clusters)
				hf[f].clusters_in = reinterpret_cast<uint32_t *>(P(o_cin)) + vbase[f];

	// ---- uploads -------------------------------------------------------------
	// the one-CTA BFS takes the fields largest first, so that the longest BFS
	// do not start in a second wave of CTAs (streamed fields, skipped there, last)
	std::vector<uint32_t> border(F);
	for(uint32_t f = 0; f < F; f++) border[f] = f;
	std::stable_sort(border.begin(), border.end(), [&](uint32_t x, uint32_t y) {
		const uint64_t kx = hf[x].stream ? 0u : reqs[x].mesh->nv, ky = hf[y].stream ? 0u : reqs[y].mesh->nv;
		return kx > ky;
	});
	cudaStream_t s = ctx->stream;
	// every staged copy below, each rounded up to 16 bytes
	const auto a16 = [](size_t b) { return align_up(b, 16); };
	size_t pin_need = a16(sizeof(FieldDev) * F) + a16(sizeof(FieldState) * F) + 2 * a16(4 * (size_t) (F + 1)) +
	                  a16(4 * wide.size()) + a16(4 * (size_t) n_stream) + a16(4 * (size_t) F);
	pin_need += fps ? a16(4 * (size_t) fps->n_init) + a16(sizeof(FpsDev)) : a16(4 * (size_t) stot);
	if(given_tops) pin_need += a16(4 * (size_t) reqs[0].nl) + a16(4 * (size_t) reqs[0].limits[reqs[0].nl - 1]);
	st = ensure_pin(ctx, pin_need);
	if(st != GP_OK) return st;
	GP_CUDA(ctx, cudaStreamSynchronize(s));  // the staging buffer may still feed a previous call
	char *pin = static_cast<char *>(ctx->pin);
	size_t po = 0;
	auto stage_copy = [&](size_t dst_off, const void *src, size_t bytes) -> cudaError_t {
		std::memcpy(pin + po, src, bytes);
		cudaError_t e = cudaMemcpyAsync(P(dst_off), pin + po, bytes, cudaMemcpyHostToDevice, s);
		po = align_up(po + bytes, 16);
		return e;
	};
	GP_CUDA(ctx, stage_copy(o_fields, hf.data(), sizeof(FieldDev) * F));
	GP_CUDA(ctx, stage_copy(o_state, hs.data(), sizeof(FieldState) * F));
	GP_CUDA(ctx, stage_copy(o_base, base.data(), 4 * (F + 1)));
	GP_CUDA(ctx, stage_copy(o_vbase, vbase.data(), 4 * (F + 1)));
	if(!wide.empty()) GP_CUDA(ctx, stage_copy(o_wide, wide.data(), 4 * wide.size()));
	if(n_stream) GP_CUDA(ctx, stage_copy(o_sids, sids.data(), 4 * (size_t) n_stream));
	GP_CUDA(ctx, stage_copy(o_border, border.data(), 4 * (size_t) F));
	if(fps)
	{
		// the seeds; the field's source count starts at n_init and grows on the device
		GP_CUDA(ctx, stage_copy(o_src, reqs[0].src, 4 * (size_t) fps->n_init));
		FpsDev fd{};
		fd.ns = fps->n_init;
		fd.ns_max = reqs[0].ns;
		fd.max_dist = INFINITY;
		fd.first = 0xFFFFFFFFu;
		GP_CUDA(ctx, stage_copy(o_fps, &fd, sizeof(fd)));
	}
	else if(!src_dev)
	{
		std::vector<uint32_t> all(stot);
		for(uint32_t f = 0; f < F; f++) std::memcpy(all.data() + sbase[f], reqs[f].src, 4 * (size_t) reqs[f].ns);
		GP_CUDA(ctx, stage_copy(o_src, all.data(), 4 * stot));
	}
	if(given_tops)
	{
		const Req &r = reqs[0];
		GP_CUDA(ctx, stage_copy(o_lim, r.limits, 4 * (size_t) r.nl));
		GP_CUDA(ctx, stage_copy(o_sorted, r.sorted, 4 * (size_t) r.limits[r.nl - 1]));
	}
	if(clusters)
		for(uint32_t f = 0; f < F; f++)
			if(reqs[f].clusters)
			{
				const size_t bytes = 4 * (size_t) reqs[f].mesh->nv;
				uint32_t *dst = reinterpret_cast<uint32_t *>(P(o_cin)) + vbase[f];
				GP_CUDA(ctx, cudaMemcpyAsync(dst, reqs[f].clusters, bytes,
				                             out_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
			}
	uint64_t h2d = po, d2h = 0;
	if(clusters && !out_dev)
		for(uint32_t f = 0; f < F; f++)
			if(reqs[f].clusters) h2d += 4ull * reqs[f].mesh->nv;
	GP_CUDA(ctx, cudaStreamSynchronize(s));  // the staging buffer is reused by the next call

	FieldDev *dF = reinterpret_cast<FieldDev *>(P(o_fields));
	FieldState *dS = reinterpret_cast<FieldState *>(P(o_state));
	GridSync *dSync = reinterpret_cast<GridSync *>(P(o_sync));
	const uint32_t *dBase = reinterpret_cast<const uint32_t *>(P(o_base));
	const uint32_t *dVbase = reinterpret_cast<const uint32_t *>(P(o_vbase));

	// ---- device work ---------------------------------------------------------
	// (captured into the plan's graph instead of run, when planning)
	const float *model = ctx->model;
	if(plan && model)
	{
		GP_CUDA(ctx, cudaMemcpyAsync(P(o_model), model, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToDevice, s));
		GP_CUDA(ctx, cudaStreamSynchronize(s));
		model = reinterpret_cast<const float *>(P(o_model));
	}
	const int kv = (f64 ? 2 : 0) + (clusters ? 1 : 0);
	gp_call_stats cs{};
	cs.n_fields = F;
	auto record = [&](cudaEvent_t ev) { return plan ? cudaSuccess : cudaEventRecord(ev, s); };
	auto device_work = [&]() -> gp_status {
	if(plan || fps) GP_CUDA(ctx, cudaMemsetAsync(dS, 0, sizeof(FieldState) * F, s));
	GP_CUDA(ctx, cudaMemsetAsync(dSync, 0, 2 * sizeof(GridSync), s));
	GP_CUDA(ctx, record(ctx->ev0));
	GP_CUDA(ctx, record(ctx->ph[0]));
	if(!given_tops)
	{
		GP_CUDA(ctx, launch_bfs_setup(dF, dS, dVbase, F, (uint32_t) vtot, s));
		if(!wide.empty())
		{
			GP_CUDA(ctx, launch_toplesets_wide(dF, dS, reinterpret_cast<const uint32_t *>(P(o_wide)),
			                                   (uint32_t) wide.size(), reinterpret_cast<uint32_t *>(P(o_wbar)),
			                                   reinterpret_cast<uint32_t *>(P(o_wtot)), (uint32_t) ctx->bfs_wide_ctas, s));
			cs.launches += 1;
		}
		GP_CUDA(ctx, launch_toplesets(dF, dS, F, &dSync->count, (uint32_t) ctx->bfs_ctas,
		                              reinterpret_cast<const uint32_t *>(P(o_border)), s));
		cs.launches += (vtot ? 1 : 0) + 2;
	}
	GP_CUDA(ctx, record(ctx->ph[1]));
	const bool learned = stage == Stage::ptp && o.schedule == GP_SCHED_LEARNED && model;
	float *dfeat = reinterpret_cast<float *>(P(o_feat));
	if(stage == Stage::features || learned)
	{
		GP_CUDA(ctx, launch_field_features(dF, dS, F, dfeat, s));
		cs.launches += 1;
	}
	if(stage == Stage::ptp)
	{
		// the CSR fan only where a row can outgrow a fan8 row (FP64 always)
		const bool csr = f64 || std::any_of(reqs, reqs + F, [](const Req &r) { return r.mesh->dev.max_fan > 7; });
		GP_CUDA(ctx, launch_renumber_batch(dF, dS, dBase, F, (uint32_t) tot, reinterpret_cast<uint32_t *>(P(o_cnt)),
		                                   reinterpret_cast<uint32_t *>(P(o_scan)), f64, clusters, csr, !given_tops, s));
		cs.launches += (csr ? 2 + scan_launches(tot) : 1) + (given_tops ? 2 : 0);
		GP_CUDA(ctx, record(ctx->ph[2]));
		// FP64 fields leave the one-CTA launch early: GB300's FP64 pipe retires
		// ~2 FMAs per clock per SM, so one CTA is throughput-bound on one SM
		// (icosphere L6: 37.8 ms at 4096, 8.9 ms at <= 256)
		const uint32_t lw = o.local_window ? o.local_window : (f64 ? LOCAL_WINDOW_F64 : LOCAL_WINDOW_F32);
		uint32_t *pbig = nullptr, *perm = nullptr;
		if(learned)
		{
			pbig = reinterpret_cast<uint32_t *>(P(o_pbig));
			perm = reinterpret_cast<uint32_t *>(P(o_perm));
			float *pred = reinterpret_cast<float *>(P(o_pred));
			GP_CUDA(ctx, mlp_infer_bf16_device(model, dfeat, (int) F, pred, s));
			GP_CUDA(ctx, launch_plan(dF, dS, F, pred, lw, pbig, reinterpret_cast<float *>(P(o_cost)), perm, s));
			cs.launches += 2;
		}
		GP_CUDA(ctx, launch_classify(dF, dS, F, lw, pbig, s));
		GP_CUDA(ctx, launch_ptp_local(dF, dS, F, reinterpret_cast<uint32_t *>(P(o_queue)),
		                              (uint32_t) ctx->local_ctas[kv], lw, perm, f64, clusters, s));
		GP_CUDA(ctx, record(ctx->ph[3]));
		ctx->grid_ctas = ctas;
		const uint32_t qmax = (uint32_t) ctx->queue_ctas[kv];
		const uint32_t qctas = o.ctas ? std::min<uint32_t>(o.ctas, qmax) : qmax;
		QCtl *dctl = reinterpret_cast<QCtl *>(P(o_qctl));
		GP_CUDA(ctx, launch_ptp_queue(dF, dS, F, reinterpret_cast<QField *>(P(o_qf)), reinterpret_cast<QLine *>(P(o_qcur)),
		                              reinterpret_cast<QLine *>(P(o_qdone)), reinterpret_cast<QLine *>(P(o_qsd)), dctl,
		                              qctas, n_stream ? GP_GRID_LOCKSTEP : o.grid_kernel,
		                              o.queue_min ? o.queue_min : QUEUE_MIN_DEFAULT, o.queue_tile, f64, clusters, s));
		GP_CUDA(ctx, launch_ptp(dF, dS, F, reinterpret_cast<uint32_t *>(P(o_notok)),
		                        reinterpret_cast<uint32_t *>(P(o_bar)), ctas, f64, clusters, ctx->steps,
		                        ctx->steps_cap, dctl, ctx->dbg_spin, ctx->dbg_phantom,
		                        reinterpret_cast<const uint32_t *>(P(o_sids)), n_stream, workers,
		                        reinterpret_cast<unsigned long long *>(P(o_sprog)),
		                        reinterpret_cast<unsigned long long *>(P(o_snap)), s));
		GP_CUDA(ctx, record(ctx->ph[4]));
		FpsDev *dfps = fps ? reinterpret_cast<FpsDev *>(P(o_fps)) : nullptr;
		GP_CUDA(ctx, launch_gather_batch(dF, dS, dBase, F, (uint32_t) tot, f64, clusters, s,
		                                 dfps ? &dfps->amax : nullptr, o.normalize != 0));
		if(o.normalize)
		{
			GP_CUDA(ctx, launch_normalize_batch(dF, dS, dBase, F, (uint32_t) tot, out_type == GP_F64, s));
			cs.launches += 1;
		}
		// classify, one-CTA sweeps, queue setup + queue kernel, lockstep (and with
		// streamed fields the plain launch that resumes after it), gather
		cs.launches += 6 + (n_stream ? 1 : 0);
	}
	else
		for(int k = 2; k < 5; k++) GP_CUDA(ctx, record(ctx->ph[k]));
	GP_CUDA(ctx, record(ctx->ph[5]));
	GP_CUDA(ctx, record(ctx->ev1));
	return GP_OK;
	};
	if(plan)
	{
		plan->n_fields = F;
		plan->state = dS;
		plan->ctl = reinterpret_cast<QCtl *>(P(o_qctl));
		plan->bar = reinterpret_cast<uint32_t *>(P(o_bar));
		plan->sync = dSync;
		GP_CUDA(ctx, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
		st = device_work();
		cudaGraph_t g = nullptr;
		const cudaError_t e = cudaStreamEndCapture(s, &g);
		if(st != GP_OK)
		{
			if(g) cudaGraphDestroy(g);
			return st;
		}
		GP_CUDA(ctx, e);
		plan->graph = g;
		GP_CUDA(ctx, cudaGraphInstantiate(&plan->exec, g, 0));
		return GP_OK;
	}
	if(fps)
	{
		// farthest-point sampling: every sample's work enqueued back to back;
		// with a radius the host looks at the device's stop flag every 8
		// samples, else only at the end
		FpsDev *dfps = reinterpret_cast<FpsDev *>(P(o_fps));
		uint32_t *dsamp = reinterpret_cast<uint32_t *>(P(o_src));
		const FpsErr fe{dSync, reinterpret_cast<const uint32_t *>(P(o_bar)),
		                reinterpret_cast<const QCtl *>(P(o_qctl)), dS,
		                wide.empty() ? nullptr : reinterpret_cast<const uint32_t *>(P(o_wbar))};
		const uint32_t chunk = fps->radio > 0 ? 8u : std::max(fps->n_iter, 1u);
		GP_CUDA(ctx, cudaEventRecord(ctx->fps0, s));
		for(uint32_t it = 0; it < fps->n_iter;)
		{
			const uint32_t n = std::min(chunk, fps->n_iter - it);
			for(uint32_t k = 0; k < n; k++)
			{
				GP_CUDA(ctx, launch_fps_sources(dF, dfps, s));
				st = device_work();
				if(st != GP_OK) return st;
				GP_CUDA(ctx, launch_fps_append(hf[0].dist_out, out_type == GP_F64, reqs[0].mesh->nv, dfps, dsamp,
				                               fps->radio, fe, s));
			}
			it += n;
			if(it < fps->n_iter)
			{
				uint32_t stop = 0;
				GP_CUDA(ctx, cudaMemcpyAsync(&stop, &dfps->stop, 4, cudaMemcpyDeviceToHost, s));
				GP_CUDA(ctx, cudaStreamSynchronize(s));
				if(stop) break;
			}
		}
		GP_CUDA(ctx, cudaEventRecord(ctx->fps1, s));
	}
	else
	{
		st = device_work();
		if(st != GP_OK) return st;
	}

	// ---- downloads -------------------------------------------------------------
	GridSync hsync[2];
	GP_CUDA(ctx, cudaMemcpyAsync(hsync, dSync, sizeof(hsync), cudaMemcpyDeviceToHost, s));
	GP_CUDA(ctx, cudaMemcpyAsync(hs.data(), dS, sizeof(FieldState) * F, cudaMemcpyDeviceToHost, s));
	d2h += sizeof(hsync) + sizeof(FieldState) * F;
	if(stage == Stage::ptp && !out_dev && !fps)
		for(uint32_t f = 0; f < F; f++)
			d2h += (uint64_t) reqs[f].mesh->nv * (osz + (reqs[f].clusters ? 4 : 0));
	FpsDev hfps{};
	if(fps)
	{
		GP_CUDA(ctx, cudaMemcpyAsync(&hfps, P(o_fps), sizeof(hfps), cudaMemcpyDeviceToHost, s));
		GP_CUDA(ctx, cudaStreamSynchronize(s));
		if(hfps.ns > fps->n_init)
			GP_CUDA(ctx, cudaMemcpyAsync(fps->samples + fps->n_init, reinterpret_cast<uint32_t *>(P(o_src)) + fps->n_init,
			                             4 * (size_t) (hfps.ns - fps->n_init), cudaMemcpyDeviceToHost, s));
		d2h += sizeof(hfps) + 4 * (size_t) (hfps.ns - fps->n_init);
		fps->n_out = hfps.ns;
		fps->max_dist = hfps.max_dist;
	}
	if(stage == Stage::ptp && !out_dev && !fps)
	{
		// the fields' outputs lie back to back in the workspace; runs of fields
		// whose host arrays also lie back to back go down in one copy
		for(uint32_t f0 = 0; f0 < F;)
		{
			uint32_t f1 = f0 + 1;
			while(f1 < F && static_cast<char *>(reqs[f1].dist) ==
			                    static_cast<char *>(reqs[f1 - 1].dist) + (size_t) reqs[f1 - 1].mesh->nv * osz)
				f1++;
			GP_CUDA(ctx, cudaMemcpyAsync(reqs[f0].dist, P(o_out) + (size_t) vbase[f0] * osz,
			                             (size_t) (vbase[f1] - vbase[f0]) * osz, cudaMemcpyDeviceToHost, s));
			f0 = f1;
		}
		for(uint32_t f = 0; f < F; f++)
			if(reqs[f].clusters)
				GP_CUDA(ctx, cudaMemcpyAsync(reqs[f].clusters, reinterpret_cast<uint32_t *>(P(o_cout)) + vbase[f],
				                             4 * (size_t) reqs[f].mesh->nv, cudaMemcpyDeviceToHost, s));
	}
	GP_CUDA(ctx, cudaStreamSynchronize(s));
	uint32_t ferr = 0;
	for(uint32_t f = 0; f < F; f++) ferr |= hs[f].status;
	QCtl hctl{};
	if(stage == Stage::ptp)
	{
		uint32_t gb[GRID_BAR_WORDS];
		GP_CUDA(ctx, cudaMemcpy(gb, P(o_bar), sizeof(gb), cudaMemcpyDeviceToHost));
		GP_CUDA(ctx, cudaMemcpy(&hctl, P(o_qctl), sizeof(hctl), cudaMemcpyDeviceToHost));
		ferr |= gb[2] | gb[BAR_RESUME + 2] | hctl.err;
	}
	if(!wide.empty())
	{
		uint32_t wb[4];
		GP_CUDA(ctx, cudaMemcpy(wb, P(o_wbar), sizeof(wb), cudaMemcpyDeviceToHost));
		ferr |= wb[2];
	}
	st = map_dev_err(ctx, hsync[0].err | hsync[1].err | ferr | hfps.err, stage == Stage::ptp ? "ptp" : "toplesets");
	if(st != GP_OK) return st;
	float ms = 0.f;
	GP_CUDA(ctx, cudaEventElapsedTime(&ms, fps ? ctx->fps0 : ctx->ev0, fps ? ctx->fps1 : ctx->ev1));
	if(seconds) *seconds = ms * 1e-3;
	{
		float pm[5];
		for(int k = 0; k < 5; k++) GP_CUDA(ctx, cudaEventElapsedTime(&pm[k], ctx->ph[k], ctx->ph[k + 1]));
		cs.ms_toplesets = pm[0];
		cs.ms_renumber = pm[1];
		cs.ms_local = pm[2];
		cs.ms_grid = pm[3];
		cs.ms_gather = pm[4];
		for(uint32_t f = 0; f < F; f++)
		{
			if(hs[f].big)
			{
				cs.fields_grid++;
				cs.relax_grid += hs[f].relax;
			}
			else cs.relax_local += hs[f].relax;
		}
		uint32_t hbar[GRID_BAR_WORDS] = {};
		if(stage == Stage::ptp)
			GP_CUDA(ctx, cudaMemcpy(hbar, P(o_bar), sizeof(hbar), cudaMemcpyDeviceToHost));
		cs.grid_kernel = hctl.mode;
		cs.fields_streamed = n_stream;
		// a streaming launch and the launch that resumes after it count apart
		const uint32_t *rb = hbar + BAR_RESUME;
		cs.sweeps_grid = hctl.mode == GRID_QUEUE ? hctl.progress : hbar[3] + rb[3];
		cs.skip_grid = hctl.mode == GRID_QUEUE
		                   ? 0
		                   : (hbar[4] | (uint64_t) hbar[5] << 32) + (rb[4] | (uint64_t) rb[5] << 32);
		cs.h2d_bytes = h2d;
		cs.d2h_bytes = d2h + (stage == Stage::ptp ? 2 * sizeof(hbar) + sizeof(hctl) : 0);
		ctx->last = cs;
	}
	for(uint32_t f = 0; f < F; f++)
		if(reqs[f].stats)
		{
			reqs[f].stats->n_iter = hs[f].n_iter;
			reqs[f].stats->n_limits = hs[f].n_limits;
			reqs[f].stats->relaxations = hs[f].relax;
			reqs[f].stats->seconds = ms * 1e-3;
		}

	if(stage == Stage::features && features)
		GP_CUDA(ctx, cudaMemcpy(features, P(o_feat), sizeof(float) * F * MLP_IN, cudaMemcpyDeviceToHost));
	if(stage == Stage::toplesets && top)
	{
		const Req &r = reqs[0];
		const uint32_t nl = hs[0].n_limits;
		if(top->n_limits) *top->n_limits = nl;
		std::vector<uint32_t> lim(nl);
		if(nl) GP_CUDA(ctx, cudaMemcpy(lim.data(), P(o_lim), 4 * (size_t) nl, cudaMemcpyDeviceToHost));
		const uint32_t nr = nl ? lim[nl - 1] : 0;
		if(top->rings)
			GP_CUDA(ctx, cudaMemcpy(top->rings, P(o_ring), 4 * (size_t) r.mesh->nv, cudaMemcpyDeviceToHost));
		if(nl > top->cap_limits || nr > top->cap_sorted)
		{
			set_err(ctx, "toplesets: need %u limits and %u sorted entries", nl, nr);
			return GP_ERR_CAPACITY;
		}
		if(top->limits && nl) std::memcpy(top->limits, lim.data(), 4 * (size_t) nl);
		if(top->sorted && nr) GP_CUDA(ctx, cudaMemcpy(top->sorted, P(o_sorted), 4 * (size_t) nr, cudaMemcpyDeviceToHost));
	}
	return GP_OK;
}

} // namespace

namespace gp {
const MeshDev *mesh_dev(const gp_mesh *mesh) { return mesh ? &mesh->dev : nullptr; }
int mesh_device(const gp_mesh *mesh) { return mesh && mesh->ctx ? mesh->ctx->device : -1; }
} // namespace gp

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char *gp_status_str(gp_status s)
{
	switch(s)
	{
		case GP_OK: return "ok";
		case GP_ERR_INVALID_ARG: return "invalid argument";
		case GP_ERR_NONMANIFOLD: return "star walk does not close";
		case GP_ERR_NO_CONVERGENCE: return "no convergence";
		case GP_ERR_DEVICE_TIMEOUT: return "device wait timed out";
		case GP_ERR_CUDA: return "CUDA error";
		case GP_ERR_NO_DEVICE: return "no usable CUDA device";
		case GP_ERR_OUT_OF_MEMORY: return "out of memory";
		case GP_ERR_CAPACITY: return "buffer too small";
	}
	return "unknown status";
}

namespace gp {
namespace {

// Unique id of the calling thread's current CUDA context (cuCtxGetId), or 0
// when it cannot be told.  The driver functions are found through the runtime
// (no link against the driver library).  A device reset destroys the primary
// context; the next runtime call makes a new one with a new id.
unsigned long long current_ctx_id()
{
	static PFN_cuCtxGetCurrent_v4000 get_cur = nullptr;
	static PFN_cuCtxGetId_v12000 get_id = nullptr;
	static std::once_flag once;
	std::call_once(once, [] {
		cudaDriverEntryPointQueryResult q{};
		void *p = nullptr;
		if(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) == cudaSuccess &&
		   q == cudaDriverEntryPointSuccess)
			get_cur = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(p);
		p = nullptr;
		if(cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
		   q == cudaDriverEntryPointSuccess)
			get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(p);
		cudaGetLastError();
	});
	if(!get_cur || !get_id) return 0;
	CUcontext c = nullptr;
	unsigned long long id = 0;
	if(get_cur(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
	return id;
}

// ctx's handles still belong to its device's current context (no device reset since)
bool ctx_alive(const gp_ctx *ctx)
{
	if(cudaSetDevice(ctx->device) != cudaSuccess)
	{
		cudaGetLastError();
		return false;
	}
	const unsigned long long id = current_ctx_id();
	return !id || !ctx->cu_id || id == ctx->cu_id;
}

} // namespace
} // namespace gp

int gp_ctx_valid(const gp_ctx *ctx) { return ctx && ctx_alive(ctx) ? 1 : 0; }

gp_status gp_ctx_create(int device, gp_ctx **out)
{
	if(!out) return GP_ERR_INVALID_ARG;
	*out = nullptr;
	int n = 0;
	if(cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n)
	{
		cudaGetLastError();
		return GP_ERR_NO_DEVICE;
	}
	int major = 0, minor = 0;
	cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device);
	cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device);
	if(major != 10 || minor != 3) return GP_ERR_NO_DEVICE;  // built for sm_103a only
	gp_ctx *ctx = new gp_ctx;
	ctx->device = device;
	if(cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
	   cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess)
	{
		cudaGetLastError();
		delete ctx;
		return GP_ERR_CUDA;
	}
	cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
	ctx->cu_id = current_ctx_id();
	ctx->bfs_ctas = toplesets_max_ctas(device);
	ctx->bfs_wide_ctas = toplesets_wide_ctas(device);
	for(int k = 0; k < 4; k++)
	{
		ctx->ptp_ctas[k] = ptp_max_ctas(device, k >= 2, k & 1, 1);
		ctx->queue_ctas[k] = ptp_queue_max_ctas(device, k >= 2, k & 1);
		ctx->local_ctas[k] = ptp_local_max_ctas(device, k >= 2, k & 1);
	}
	for(int k = 0; k < 6; k++)
		if(cudaEventCreate(&ctx->ph[k]) != cudaSuccess) ctx->ph[k] = nullptr;
	if(cudaEventCreate(&ctx->fps0) != cudaSuccess || cudaEventCreate(&ctx->fps1) != cudaSuccess) ctx->ph[5] = nullptr;
	if(ctx->bfs_ctas <= 0 || ctx->ptp_ctas[0] <= 0 || !ctx->ph[5])
	{
		cudaGetLastError();
		gp_ctx_destroy(ctx);
		return GP_ERR_NO_DEVICE;
	}
	*out = ctx;
	return GP_OK;
}

void gp_ctx_destroy(gp_ctx *ctx)
{
	if(!ctx) return;
	if(!ctx_alive(ctx))
	{
		// the device was reset: its handles died with the old context
		delete ctx;
		return;
	}
	if(ctx->stream) cudaStreamSynchronize(ctx->stream);
	if(ctx->ws) cudaFree(ctx->ws);
	if(ctx->pin) cudaFreeHost(ctx->pin);
	if(ctx->steps) cudaFree(ctx->steps);
	if(ctx->model) cudaFree(ctx->model);
	if(ctx->ev0) cudaEventDestroy(ctx->ev0);
	if(ctx->ev1) cudaEventDestroy(ctx->ev1);
	for(int k = 0; k < 6; k++)
		if(ctx->ph[k]) cudaEventDestroy(ctx->ph[k]);
	if(ctx->fps0) cudaEventDestroy(ctx->fps0);
	if(ctx->fps1) cudaEventDestroy(ctx->fps1);
	if(ctx->stream) cudaStreamDestroy(ctx->stream);
	delete ctx;
}

const char *gp_ctx_last_error(const gp_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

gp_status gp_ctx_step_trace(gp_ctx *ctx, uint32_t cap, uint64_t *out, uint32_t *n_out)
{
	if(!ctx) return GP_ERR_INVALID_ARG;
	if(!out)
	{
		// (re)arm: record up to cap steps of the following calls' grid launches
		if(ctx->steps) cudaFree(ctx->steps);
		ctx->steps = nullptr;
		ctx->steps_cap = 0;
		if(cap)
		{
			GP_CUDA(ctx, cudaMalloc(&ctx->steps, 16 * (size_t) cap));
			ctx->steps_cap = cap;
		}
		return GP_OK;
	}
	if(!ctx->steps || !n_out) return GP_ERR_INVALID_ARG;
	const uint32_t n = std::min(cap, ctx->steps_cap);
	GP_CUDA(ctx, cudaMemcpy(out, ctx->steps, 16 * (size_t) n, cudaMemcpyDeviceToHost));
	uint32_t k = 0;
	while(k < n && out[2 * k]) k++;
	*n_out = k;
	return GP_OK;
}

gp_status gp_ctx_call_stats(const gp_ctx *ctx, gp_call_stats *out)
{
	if(!ctx || !out) return GP_ERR_INVALID_ARG;
	*out = ctx->last;
	return GP_OK;
}
void *gp_ctx_stream(gp_ctx *ctx) { return ctx ? (void *) ctx->stream : nullptr; }
size_t gp_ctx_workspace_bytes(const gp_ctx *ctx) { return ctx ? ctx->ws_bytes : 0; }

gp_status gp_ctx_device_info(const gp_ctx *ctx, int *cc, int *binary_version, int *num_sms)
{
	if(!ctx) return GP_ERR_INVALID_ARG;
	GP_CUDA(const_cast<gp_ctx *>(ctx), cudaSetDevice(ctx->device));
	int major = 0, minor = 0;
	cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, ctx->device);
	cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, ctx->device);
	if(cc) *cc = 10 * major + minor;
	if(binary_version) *binary_version = ptp_binary_version();
	if(num_sms) *num_sms = ctx->num_sms;
	return GP_OK;
}

gp_status gp_che_build(uint32_t nv, uint32_t nf, const uint32_t *VT, uint32_t *OT, uint32_t *EVT, int *manifold)
{
	// Compact half-edge opposite/extra-vertex tables with the matching order
	// and non-manifold rule of che::update_evt_ot_et (src/che.cpp:1295-1362):
	// half-edge he pairs with the first still-free prev(h) among the
	// half-edges h leaving VT[he] (in half-edge order) with VT[prev(h)] ==
	// VT[next(he)]; a border vertex whose EVT is a different border
	// half-edge is non-manifold and gets EVT = NIL.
	if((nf && (!VT || !OT)) || (nv && !EVT)) return GP_ERR_INVALID_ARG;
	const uint64_t nhe = 3ull * nf;
	if(nhe >= 0xFFFFFFFFull) return GP_ERR_INVALID_ARG;
	for(uint64_t he = 0; he < nhe; he++)
		if(VT[he] >= nv) return GP_ERR_INVALID_ARG;
	std::fill(EVT, EVT + nv, NIL);
	if(manifold) *manifold = 1;
	if(!nf) return GP_OK;
	std::vector<uint32_t> start(nv + 1, 0), byv(nhe);
	for(uint64_t he = 0; he < nhe; he++)
	{
		EVT[VT[he]] = (uint32_t) he;
		start[VT[he] + 1]++;
	}
	for(uint32_t v = 0; v < nv; v++) start[v + 1] += start[v];
	{
		std::vector<uint32_t> fill(start.begin(), start.end() - 1);
		for(uint64_t he = 0; he < nhe; he++) byv[fill[VT[he]]++] = (uint32_t) he;
	}
	std::fill(OT, OT + nhe, NIL);
	for(uint32_t he = 0; he < nhe; he++)
	{
		if(OT[he] != NIL) continue;
		const uint32_t a = VT[he], b = VT[he_next(he)];
		for(uint32_t k = start[a]; k < start[a + 1]; k++)
		{
			const uint32_t ph = he_prev(byv[k]);
			if(VT[ph] == b && OT[he] == NIL && OT[ph] == NIL)
			{
				OT[he] = ph;
				OT[ph] = he;
			}
		}
	}
	for(uint32_t he = 0; he < nhe; he++)
	{
		const uint32_t v = VT[he];
		if(OT[he] != NIL || EVT[v] == NIL) continue;
		if(OT[EVT[v]] == NIL && EVT[v] != he)
		{
			EVT[v] = NIL;
			if(manifold) *manifold = 0;
		}
		else EVT[v] = he;
	}
	return GP_OK;
}

gp_status gp_che_build_device(gp_ctx *ctx, uint32_t nv, uint32_t nf, const uint32_t *VT, uint32_t *OT, uint32_t *EVT,
                              int *manifold)
{
	if(!ctx || (nf && (!VT || !OT)) || (nv && !EVT)) return GP_ERR_INVALID_ARG;
	const uint64_t nhe = 3ull * nf;
	if(nhe >= 0x7FFFFFFFull || nv >= 0x7FFFFFFFu) return GP_ERR_CAPACITY;
	for(uint64_t he = 0; he < nhe; he++)
		if(VT[he] >= nv)
		{
			set_err(ctx, "VT[%llu] out of range", (unsigned long long) he);
			return GP_ERR_INVALID_ARG;
		}
	Carve c;
	const size_t o_vt = c.add<uint32_t>(nhe), o_ot = c.add<uint32_t>(nhe), o_evt = c.add<uint32_t>(nv);
	const size_t o_s = c.add<char>(che_build_scratch_bytes(nv, (uint32_t) nhe)), o_f = c.add<uint32_t>(4);
	gp_status st = ensure_ws(ctx, c.off);
	if(st != GP_OK) return st;
	char *W = static_cast<char *>(ctx->ws);
	cudaStream_t s = ctx->stream;
	uint32_t f[4];
	GP_CUDA(ctx, cudaMemcpyAsync(W + o_vt, VT, 4 * nhe, cudaMemcpyHostToDevice, s));
	GP_CUDA(ctx, launch_che_build(reinterpret_cast<uint32_t *>(W + o_vt), nv, (uint32_t) nhe,
	                              reinterpret_cast<uint32_t *>(W + o_ot), reinterpret_cast<uint32_t *>(W + o_evt), W + o_s,
	                              reinterpret_cast<uint32_t *>(W + o_f), s));
	GP_CUDA(ctx, cudaMemcpyAsync(f, W + o_f, sizeof(f), cudaMemcpyDeviceToHost, s));
	if(nhe) GP_CUDA(ctx, cudaMemcpyAsync(OT, W + o_ot, 4 * nhe, cudaMemcpyDeviceToHost, s));
	if(nv) GP_CUDA(ctx, cudaMemcpyAsync(EVT, W + o_evt, 4 * (size_t) nv, cudaMemcpyDeviceToHost, s));
	GP_CUDA(ctx, cudaStreamSynchronize(s));
	if(f[0] & 8u)
	{
		set_err(ctx, "an edge or border list too long for the GPU build");
		return GP_ERR_CAPACITY;
	}
	if(f[0])
	{
		set_err(ctx, "half-edge table build: bad index (err=%u)", f[0]);
		return GP_ERR_INVALID_ARG;
	}
	if(manifold) *manifold = f[1] ? 0 : 1;
	return GP_OK;
}

gp_status gp_off_read(const char *path, uint32_t *n_vertices, uint32_t *n_faces, double *xyz, uint32_t cap_vertices,
                      uint32_t *VT, uint32_t cap_faces)
{
	if(!path || !n_vertices || !n_faces) return GP_ERR_INVALID_ARG;
	std::vector<double> X;
	std::vector<uint32_t> T;
	std::string err;
	const gp_status st = off_parse(path, X, T, err);
	if(st != GP_OK) return st;
	*n_vertices = (uint32_t) (X.size() / 3);
	*n_faces = (uint32_t) (T.size() / 3);
	if(xyz)
	{
		if(cap_vertices < *n_vertices) return GP_ERR_CAPACITY;
		std::memcpy(xyz, X.data(), sizeof(double) * X.size());
	}
	if(VT)
	{
		if(cap_faces < *n_faces) return GP_ERR_CAPACITY;
		std::memcpy(VT, T.data(), sizeof(uint32_t) * T.size());
	}
	return GP_OK;
}

gp_status gp_mesh_create_off(gp_ctx *ctx, const char *path, gp_mesh **out)
{
	if(!ctx || !path || !out) return GP_ERR_INVALID_ARG;
	std::vector<double> X;
	std::vector<uint32_t> T;
	std::string err;
	const gp_status st = off_parse(path, X, T, err);
	if(st != GP_OK)
	{
		set_err(ctx, "%s", err.c_str());
		return st;
	}
	return gp_mesh_create(ctx, (uint32_t) (X.size() / 3), X.data(), (uint32_t) (T.size() / 3), T.data(), nullptr,
	                      nullptr, out);
}

gp_status gp_mesh_create(gp_ctx *ctx, uint32_t nv, const double *xyz, uint32_t nf, const uint32_t *VT,
                         const uint32_t *OT, const uint32_t *EVT, gp_mesh **out)
{
	if(!ctx || !out || !xyz || !nv || (nf && !VT)) return GP_ERR_INVALID_ARG;
	*out = nullptr;
	if((uint64_t) 3 * nf >= 0x7FFFFFFFull || nv >= 0x7FFFFFFFu)
	{
		set_err(ctx, "mesh too large");
		return GP_ERR_CAPACITY;
	}
	const uint32_t nhe = 3 * nf;
	std::vector<uint32_t> ot_b, evt_b;
	const bool build = !OT || !EVT;  // half-edge tables built on the GPU
	if(build)
	{
		for(uint32_t he = 0; he < nhe; he++)
			if(VT[he] >= nv)
			{
				set_err(ctx, "VT[%u] = %u out of range (n_vertices %u)", he, VT[he], nv);
				return GP_ERR_INVALID_ARG;
			}
	}
	else
	{
		for(uint32_t he = 0; he < nhe; he++)
			if(VT[he] >= nv || (OT[he] != NIL && OT[he] >= nhe))
			{
				set_err(ctx, "VT/OT entry %u out of range", he);
				return GP_ERR_INVALID_ARG;
			}
		for(uint32_t v = 0; v < nv; v++)
			if(EVT[v] != NIL && EVT[v] >= nhe)
			{
				set_err(ctx, "EVT[%u] out of range", v);
				return GP_ERR_INVALID_ARG;
			}
	}
	GP_CUDA(ctx, cudaSetDevice(ctx->device));
	cudaStream_t s = ctx->stream;
	// temporaries: VT, OT, EVT, counts (+flags), scan scratch, xyz, err
	Carve tc;
	const size_t t_vt = tc.add<uint32_t>(nhe), t_ot = tc.add<uint32_t>(nhe), t_evt = tc.add<uint32_t>(nv);
	const size_t t_cnt = tc.add<uint32_t>(nv + 1), t_flags = tc.add<uint32_t>(nv);
	const size_t t_scan = tc.add<uint32_t>(scan_tmp_words(nv)), t_xyz = tc.add<double>(3 * (size_t) nv);
	const size_t t_err = tc.add<uint32_t>(4), t_acc = tc.add<double>(8);
	const size_t t_che = build ? tc.add<char>(che_build_scratch_bytes(nv, nhe)) : 0, t_cf = tc.add<uint32_t>(4);
	gp_status st = ensure_ws(ctx, tc.off);
	if(st != GP_OK) return st;
	char *T = static_cast<char *>(ctx->ws);
	GP_CUDA(ctx, cudaMemcpyAsync(T + t_vt, VT, 4 * (size_t) nhe, cudaMemcpyHostToDevice, s));
	if(build)
	{
		uint32_t cf[4];
		GP_CUDA(ctx, launch_che_build(reinterpret_cast<uint32_t *>(T + t_vt), nv, nhe, reinterpret_cast<uint32_t *>(T + t_ot),
		                              reinterpret_cast<uint32_t *>(T + t_evt), T + t_che,
		                              reinterpret_cast<uint32_t *>(T + t_cf), s));
		GP_CUDA(ctx, cudaMemcpyAsync(cf, T + t_cf, sizeof(cf), cudaMemcpyDeviceToHost, s));
		GP_CUDA(ctx, cudaStreamSynchronize(s));
		if(cf[0] & ~8u)
		{
			set_err(ctx, "half-edge table build: bad index (err=%u)", cf[0]);
			return GP_ERR_INVALID_ARG;
		}
		if(cf[0] & 8u)
		{
			// an edge shared by more than 32 half-edges, or a vertex with more
			// than 32 border half-edges: the host builds the tables
			ot_b.resize(nhe);
			evt_b.resize(nv);
			gp_che_build(nv, nf, VT, ot_b.data(), evt_b.data(), nullptr);
			GP_CUDA(ctx, cudaMemcpyAsync(T + t_ot, ot_b.data(), 4 * (size_t) nhe, cudaMemcpyHostToDevice, s));
			GP_CUDA(ctx, cudaMemcpyAsync(T + t_evt, evt_b.data(), 4 * (size_t) nv, cudaMemcpyHostToDevice, s));
		}
	}
	else
	{
		GP_CUDA(ctx, cudaMemcpyAsync(T + t_ot, OT, 4 * (size_t) nhe, cudaMemcpyHostToDevice, s));
		GP_CUDA(ctx, cudaMemcpyAsync(T + t_evt, EVT, 4 * (size_t) nv, cudaMemcpyHostToDevice, s));
	}
	GP_CUDA(ctx, cudaMemcpyAsync(T + t_xyz, xyz, 24 * (size_t) nv, cudaMemcpyHostToDevice, s));
	GP_CUDA(ctx, cudaMemsetAsync(T + t_err, 0, 16, s));
	uint32_t *dvt = reinterpret_cast<uint32_t *>(T + t_vt), *dot = reinterpret_cast<uint32_t *>(T + t_ot);
	uint32_t *devt = reinterpret_cast<uint32_t *>(T + t_evt), *dflags = reinterpret_cast<uint32_t *>(T + t_flags);
	uint32_t *dcnt = reinterpret_cast<uint32_t *>(T + t_cnt), *derr = reinterpret_cast<uint32_t *>(T + t_err);
	GP_CUDA(ctx, launch_fan_count(dvt, dot, devt, nv, nhe, dflags, derr, s));
	GP_CUDA(ctx, launch_strip_flags(dflags, dcnt, nv, s));
	GP_CUDA(ctx, launch_scan_u32(dcnt, dcnt, nv, reinterpret_cast<uint32_t *>(T + t_scan), s));
	GP_CUDA(ctx, launch_max_u32(dflags, nv, derr + 1, s));
	uint32_t h[2] = {0, 0}, n_fan = 0;
	GP_CUDA(ctx, cudaMemcpyAsync(h, derr, 8, cudaMemcpyDeviceToHost, s));
	GP_CUDA(ctx, cudaMemcpyAsync(&n_fan, dcnt + nv, 4, cudaMemcpyDeviceToHost, s));
	GP_CUDA(ctx, cudaStreamSynchronize(s));
	if(h[0])
	{
		set_err(ctx, "mesh: a star walk does not close (err=%u)", h[0]);
		return h[0] & DEV_ERR_WALK ? GP_ERR_NONMANIFOLD : GP_ERR_INVALID_ARG;
	}
	gp_mesh *m = new gp_mesh;
	m->ctx = ctx;
	m->device = ctx->device;
	m->cu_id = ctx->cu_id;
	m->nv = nv;
	m->nf = nf;
	Carve mc;
	const size_t m_pos = mc.add<float4>(nv), m_posd = mc.add<double>(4 * (size_t) nv);
	const size_t m_off = mc.add<uint32_t>(nv + 1), m_fan = mc.add<uint32_t>(n_fan);
	const size_t m_fan8 = mc.add<uint4>(2 * (size_t) nv);
	cudaError_t e = cudaMalloc(&m->block, mc.off);
	if(e != cudaSuccess)
	{
		delete m;
		set_err(ctx, "cudaMalloc mesh: %s", cudaGetErrorString(e));
		return GP_ERR_OUT_OF_MEMORY;
	}
	char *B = static_cast<char *>(m->block);
	m->dev.pos = reinterpret_cast<float4 *>(B + m_pos);
	m->dev.posd = reinterpret_cast<double *>(B + m_posd);
	m->dev.fan_off = reinterpret_cast<uint32_t *>(B + m_off);
	m->dev.fan = reinterpret_cast<uint32_t *>(B + m_fan);
	m->dev.fan8 = reinterpret_cast<uint4 *>(B + m_fan8);
	m->dev.nv = nv;
	m->dev.n_fan = n_fan;
	m->dev.max_fan = h[1];
	uint32_t *doff = const_cast<uint32_t *>(m->dev.fan_off);
	e = cudaMemcpyAsync(doff, dcnt, 4 * ((size_t) nv + 1), cudaMemcpyDeviceToDevice, s);
	if(e == cudaSuccess) e = launch_fan_fill(dvt, dot, devt, nv, dflags, doff, const_cast<uint32_t *>(m->dev.fan), s);
	if(e == cudaSuccess) e = launch_fan8(doff, m->dev.fan, nv, const_cast<uint4 *>(m->dev.fan8), s);
	if(e == cudaSuccess)
		e = launch_pos_convert(reinterpret_cast<double *>(T + t_xyz), nv, const_cast<float4 *>(m->dev.pos),
		                       const_cast<double *>(m->dev.posd), s);
	double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
	double *dacc = reinterpret_cast<double *>(T + t_acc);
	if(e == cudaSuccess) e = cudaMemsetAsync(dacc, 0, sizeof(acc), s);
	if(e == cudaSuccess) e = launch_mesh_stats(dvt, dot, m->dev.pos, nf, dacc, s);
	if(e == cudaSuccess) e = cudaMemcpyAsync(acc, dacc, sizeof(acc), cudaMemcpyDeviceToHost, s);
	if(e == cudaSuccess) e = cudaStreamSynchronize(s);
	if(e == cudaSuccess)
	{
		const double ne = std::max(acc[4], 1.0), mean = acc[0] / ne, var = std::max(acc[1] / ne - mean * mean, 0.0);
		const double gm = acc[2] / ne, gvar = std::max(acc[3] / ne - gm * gm, 0.0);
		m->dev.stats[0] = (float) std::log(std::max(mean, 1e-30));
		m->dev.stats[1] = (float) (mean > 0 ? std::sqrt(var) / mean : 0.0);
		m->dev.stats[2] = (float) std::sqrt(gvar);
		m->dev.stats[3] = (float) (nf ? acc[5] / nf : 0.0);
		m->dev.stats[4] = (float) (acc[7] > 0 ? acc[6] / acc[7] : 0.0);
	}
	if(e != cudaSuccess)
	{
		set_err(ctx, "mesh upload: %s", cudaGetErrorString(e));
		cudaFree(m->block);
		delete m;
		return GP_ERR_CUDA;
	}
	*out = m;
	return GP_OK;
}

void gp_mesh_destroy(gp_mesh *m)
{
	// cudaFree waits for work on the buffer; the owning gp_ctx is not
	// touched, so meshes may outlive (and be freed after) their context.  A
	// block that died with a device reset is not freed again.
	if(!m) return;
	if(m->block)
	{
		int prev = -1;
		cudaGetDevice(&prev);
		if(cudaSetDevice(m->device) == cudaSuccess)
		{
			const unsigned long long id = current_ctx_id();
			if(!id || !m->cu_id || id == m->cu_id) cudaFree(m->block);
		}
		if(prev >= 0) cudaSetDevice(prev);
		cudaGetLastError();
	}
	delete m;
}

uint32_t gp_mesh_n_vertices(const gp_mesh *m) { return m ? m->nv : 0; }
uint32_t gp_mesh_n_faces(const gp_mesh *m) { return m ? m->nf : 0; }

gp_status gp_toplesets(gp_ctx *ctx, gp_mesh *mesh, const uint32_t *sources, uint32_t n_sources, uint32_t *rings,
                       uint32_t *sorted, uint32_t cap_sorted, uint32_t *limits, uint32_t cap_limits, uint32_t *n_limits)
{
	if(!ctx || !mesh || !sources || !n_sources || !limits || !n_limits) return GP_ERR_INVALID_ARG;
	Req r{mesh, sources, n_sources, nullptr, 0, nullptr, nullptr, nullptr, nullptr};
	TopOut t{rings, sorted, cap_sorted, limits, cap_limits, n_limits};
	return run(ctx, &r, 1, nullptr, GP_F32, false, false, Stage::toplesets, &t, nullptr);
}

gp_status gp_ptp(gp_ctx *ctx, gp_mesh *mesh, const uint32_t *sources, uint32_t n_sources, const uint32_t *limits,
                 uint32_t n_limits, const uint32_t *sorted, const gp_ptp_opts *opts, void *dist, gp_dtype dist_type,
                 uint32_t *clusters, gp_ptp_stats *stats)
{
	if(!ctx || !mesh || !dist) return GP_ERR_INVALID_ARG;
	if((limits == nullptr) != (sorted == nullptr)) return GP_ERR_INVALID_ARG;
	Req r{mesh, sources, n_sources, limits, n_limits, sorted, dist, clusters, stats};
	return run(ctx, &r, 1, opts, dist_type, false, false, Stage::ptp, nullptr, nullptr);
}

gp_status gp_ptp_batch(gp_ctx *ctx, const gp_field *fields, uint32_t n_fields, const gp_ptp_opts *opts,
                       gp_dtype dist_type, uint32_t flags, double *seconds)
{
	if(!ctx || (n_fields && !fields)) return GP_ERR_INVALID_ARG;
	std::vector<Req> reqs(n_fields);
	for(uint32_t f = 0; f < n_fields; f++)
		reqs[f] = Req{fields[f].mesh, fields[f].sources, fields[f].n_sources, nullptr, 0, nullptr,
		              fields[f].dist, fields[f].clusters, fields[f].stats};
	const bool dev = (flags & GP_BATCH_DEVICE_POINTERS) != 0;
	const uint32_t chunk = ptp_grid_max_fields();
	double total = 0;
	for(uint32_t f0 = 0; f0 < n_fields; f0 += chunk)
	{
		double sec = 0;
		const gp_status st = run(ctx, reqs.data() + f0, std::min(chunk, n_fields - f0), opts, dist_type, dev, dev,
		                         Stage::ptp, nullptr, &sec);
		if(st != GP_OK) return st;
		total += sec;
	}
	if(seconds) *seconds = total;
	return GP_OK;
}

gp_status gp_ptp_autotune(gp_ctx *ctx, const gp_field *fields, uint32_t n_fields, gp_dtype dist_type,
                          uint32_t flags, gp_ptp_opts *opts, uint32_t reps)
{
	if(!ctx || !opts || !n_fields || !fields) return GP_ERR_INVALID_ARG;
	reps = std::max<uint32_t>(reps, 1);
	auto timed = [&](const gp_ptp_opts &o, double &best) -> gp_status {
		best = INFINITY;
		for(uint32_t r = 0; r < reps; r++)
		{
			double sec = 0;
			const gp_status st = gp_ptp_batch(ctx, fields, n_fields, &o, dist_type, flags, &sec);
			if(st != GP_OK) return st;
			best = std::min(best, sec);
		}
		return GP_OK;
	};
	// coordinate search: the one-CTA window first (lockstep grid), then the
	// grid launch and its tile at that window.  Every candidate runs the same
	// sweeps, so the results do not depend on the choice.
	gp_ptp_opts cur = *opts, best_o = *opts;
	double best = INFINITY, t = 0;
	cur.grid_kernel = GP_GRID_LOCKSTEP;
	const bool f64 = opts->precision == GP_F64;
	// (benchmark batch: 128 -> 82.6 ms per call, 1024 -> 82.9, 2048 -> 83.1:
	// in a large batch the grid launch takes almost every field at no cost)
	const std::initializer_list<uint32_t> windows32 = {128u, 256u, 512u, 1024u, 2048u, 4096u, 8192u, 16384u};
	const std::initializer_list<uint32_t> windows64 = {64u, 256u, 1024u, 4096u};
	for(uint32_t lw : f64 ? windows64 : windows32)
	{
		cur.local_window = lw;
		const gp_status st = timed(cur, t);
		if(st != GP_OK) return st;
		if(t < best)
		{
			best = t;
			best_o = cur;
		}
	}
	cur = best_o;
	cur.grid_kernel = GP_GRID_QUEUE;
	for(uint32_t tile : {64u, 128u, 256u})
	{
		cur.queue_tile = tile;
		const gp_status st = timed(cur, t);
		if(st != GP_OK) return st;
		if(t < best)
		{
			best = t;
			best_o = cur;
		}
	}
	*opts = best_o;
	return GP_OK;
}

gp_status gp_plan_create(gp_ctx *ctx, const gp_field *fields, uint32_t n_fields, const gp_ptp_opts *opts,
                         gp_dtype dist_type, gp_plan **out)
{
	if(!ctx || !fields || !n_fields || !out) return GP_ERR_INVALID_ARG;
	*out = nullptr;
	if(n_fields > ptp_grid_max_fields())
	{
		set_err(ctx, "a plan holds at most %u fields", ptp_grid_max_fields());
		return GP_ERR_CAPACITY;
	}
	std::vector<Req> reqs(n_fields);
	for(uint32_t f = 0; f < n_fields; f++)
	{
		if(fields[f].clusters)
		{
			set_err(ctx, "field %u: labels are not supported by plans", f);
			return GP_ERR_INVALID_ARG;
		}
		reqs[f] = Req{fields[f].mesh, fields[f].sources, fields[f].n_sources, nullptr, 0, nullptr,
		              fields[f].dist, nullptr, nullptr};
	}
	gp_plan *p = new gp_plan;
	p->ctx = ctx;
	const gp_status st = run(ctx, reqs.data(), n_fields, opts, dist_type, true, true, Stage::ptp, nullptr, nullptr,
	                         nullptr, p);
	if(st != GP_OK)
	{
		gp_plan_destroy(p);
		return st;
	}
	*out = p;
	return GP_OK;
}

gp_status gp_plan_launch(gp_plan *plan, void *stream)
{
	if(!plan || !plan->exec) return GP_ERR_INVALID_ARG;
	gp_ctx *ctx = plan->ctx;
	GP_CUDA(ctx, cudaGraphLaunch(plan->exec, stream ? static_cast<cudaStream_t>(stream) : ctx->stream));
	return GP_OK;
}

gp_status gp_plan_wait(gp_plan *plan, void *stream, gp_ptp_stats *stats)
{
	if(!plan) return GP_ERR_INVALID_ARG;
	gp_ctx *ctx = plan->ctx;
	cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
	const uint32_t F = plan->n_fields;
	std::vector<FieldState> hs(F);
	GridSync hsync[2];
	uint32_t hbar[GRID_BAR_WORDS];
	QCtl hctl{};
	GP_CUDA(ctx, cudaMemcpyAsync(hs.data(), plan->state, sizeof(FieldState) * F, cudaMemcpyDeviceToHost, s));
	GP_CUDA(ctx, cudaMemcpyAsync(hsync, plan->sync, sizeof(hsync), cudaMemcpyDeviceToHost, s));
	GP_CUDA(ctx, cudaMemcpyAsync(hbar, plan->bar, sizeof(hbar), cudaMemcpyDeviceToHost, s));
	GP_CUDA(ctx, cudaMemcpyAsync(&hctl, plan->ctl, sizeof(hctl), cudaMemcpyDeviceToHost, s));
	GP_CUDA(ctx, cudaStreamSynchronize(s));
	uint32_t err = hsync[0].err | hsync[1].err | hbar[2] | hbar[BAR_RESUME + 2] | hctl.err;
	for(uint32_t f = 0; f < F; f++)
	{
		err |= hs[f].status;
		if(stats)
		{
			stats[f].n_iter = hs[f].n_iter;
			stats[f].n_limits = hs[f].n_limits;
			stats[f].relaxations = hs[f].relax;
			stats[f].seconds = 0;
		}
	}
	return map_dev_err(ctx, err, "plan");
}

void gp_plan_destroy(gp_plan *plan)
{
	if(!plan) return;
	if(plan->exec) cudaGraphExecDestroy(plan->exec);
	if(plan->graph) cudaGraphDestroy(plan->graph);
	if(plan->ws) cudaFree(plan->ws);
	delete plan;
}

gp_status gp_ctx_debug_barrier(gp_ctx *ctx, uint32_t spin_limit, uint32_t phantom_arrivals)
{
	if(!ctx) return GP_ERR_INVALID_ARG;
	ctx->dbg_spin = spin_limit;
	ctx->dbg_phantom = phantom_arrivals;
	return GP_OK;
}

uint32_t gp_mlp_n_params(void) { return (uint32_t) MLP_NPARAM; }

gp_status gp_ctx_set_cost_model(gp_ctx *ctx, const float *params)
{
	if(!ctx) return GP_ERR_INVALID_ARG;
	if(!params)
	{
		if(ctx->model) cudaFree(ctx->model);
		ctx->model = nullptr;
		return GP_OK;
	}
	if(!ctx->model) GP_CUDA(ctx, cudaMalloc(reinterpret_cast<void **>(&ctx->model), sizeof(float) * MLP_NPARAM));
	GP_CUDA(ctx, cudaMemcpy(ctx->model, params, sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice));
	return GP_OK;
}

gp_status gp_field_features(gp_ctx *ctx, const gp_field *fields, uint32_t n_fields, float *features)
{
	if(!ctx || !features || (n_fields && !fields)) return GP_ERR_INVALID_ARG;
	std::vector<Req> reqs(n_fields);
	for(uint32_t f = 0; f < n_fields; f++)
		reqs[f] = Req{fields[f].mesh, fields[f].sources, fields[f].n_sources, nullptr, 0, nullptr, nullptr, nullptr,
		              nullptr};
	return run(ctx, reqs.data(), n_fields, nullptr, GP_F32, false, false, Stage::features, nullptr, nullptr, features);
}

namespace {

// Device buffers of one MLP call inside the context workspace.
struct MlpBufs {
	float *X, *T, *P, *G, *M1, *M2, *work, *Y, *loss;
};

gp_status mlp_bufs(gp_ctx *ctx, uint32_t n, MlpBufs &b, uint32_t epochs = 0)
{
	Carve c;
	const size_t oX = c.add<float>((size_t) n * MLP_IN), oT = c.add<float>((size_t) n * MLP_OUT);
	const size_t oP = c.add<float>(MLP_NPARAM), oG = c.add<float>(MLP_NPARAM), oM1 = c.add<float>(MLP_NPARAM),
	             oM2 = c.add<float>(MLP_NPARAM), oW = c.add<float>(mlp_workspace_floats((int) n)),
	             oY = c.add<float>((size_t) n * MLP_OUT), oL = c.add<float>(4 + (size_t) epochs);
	gp_status st = ensure_ws(ctx, c.off);
	if(st != GP_OK) return st;
	char *W = static_cast<char *>(ctx->ws);
	b = MlpBufs{reinterpret_cast<float *>(W + oX), reinterpret_cast<float *>(W + oT), reinterpret_cast<float *>(W + oP),
	            reinterpret_cast<float *>(W + oG), reinterpret_cast<float *>(W + oM1), reinterpret_cast<float *>(W + oM2),
	            reinterpret_cast<float *>(W + oW), reinterpret_cast<float *>(W + oY), reinterpret_cast<float *>(W + oL)};
	return GP_OK;
}

} // namespace

gp_status gp_mlp_grad(gp_ctx *ctx, const float *X, const float *T, uint32_t n, const float *params, float *grads,
                      float *loss)
{
	if(!ctx || !X || !T || !n || !params || !grads || !loss) return GP_ERR_INVALID_ARG;
	MlpBufs b;
	gp_status st = mlp_bufs(ctx, n, b);
	if(st != GP_OK) return st;
	cudaStream_t s = ctx->stream;
	GP_CUDA(ctx, cudaMemcpyAsync(b.X, X, sizeof(float) * n * MLP_IN, cudaMemcpyHostToDevice, s));
	GP_CUDA(ctx, cudaMemcpyAsync(b.T, T, sizeof(float) * n * MLP_OUT, cudaMemcpyHostToDevice, s));
	GP_CUDA(ctx, cudaMemcpyAsync(b.P, params, sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice, s));
	GP_CUDA(ctx, mlp_grad_device(b.P, b.X, b.T, (int) n, b.work, b.G, b.loss, s));
	GP_CUDA(ctx, cudaMemcpyAsync(grads, b.G, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost, s));
	GP_CUDA(ctx, cudaMemcpyAsync(loss, b.loss, sizeof(float), cudaMemcpyDeviceToHost, s));
	GP_CUDA(ctx, cudaStreamSynchronize(s));
	return GP_OK;
}

gp_status gp_mlp_train(gp_ctx *ctx, const float *X, const float *T, uint32_t n, float *params, uint32_t epochs,
                       float lr, float *losses)
{
	if(!ctx || !X || !T || !n || !params) return GP_ERR_INVALID_ARG;
	MlpBufs b;
	gp_status st = mlp_bufs(ctx, n, b, epochs);
	if(st != GP_OK) return st;
	cudaStream_t s = ctx->stream;
	GP_CUDA(ctx, cudaMemcpyAsync(b.X, X, sizeof(float) * n * MLP_IN, cudaMemcpyHostToDevice, s));
	GP_CUDA(ctx, cudaMemcpyAsync(b.T, T, sizeof(float) * n * MLP_OUT, cudaMemcpyHostToDevice, s));
	GP_CUDA(ctx, cudaMemcpyAsync(b.P, params, sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice, s));
	GP_CUDA(ctx, cudaMemsetAsync(b.M1, 0, sizeof(float) * MLP_NPARAM, s));
	GP_CUDA(ctx, cudaMemsetAsync(b.M2, 0, sizeof(float) * MLP_NPARAM, s));
	float *dl = b.loss + 4;  // per-epoch losses stay on the device until the end
	for(uint32_t ep = 0; ep < epochs; ep++)
	{
		GP_CUDA(ctx, mlp_grad_device(b.P, b.X, b.T, (int) n, b.work, b.G, b.loss, s));
		if(losses) GP_CUDA(ctx, cudaMemcpyAsync(dl + ep, b.loss, sizeof(float), cudaMemcpyDeviceToDevice, s));
		GP_CUDA(ctx, mlp_adam_device(b.P, b.G, b.M1, b.M2, lr, (int) ep + 1, s));
	}
	GP_CUDA(ctx, cudaMemcpyAsync(params, b.P, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost, s));
	if(losses && epochs)
		GP_CUDA(ctx, cudaMemcpyAsync(losses, dl, sizeof(float) * epochs, cudaMemcpyDeviceToHost, s));
	GP_CUDA(ctx, cudaStreamSynchronize(s));
	return GP_OK;
}

gp_status gp_mlp_infer(gp_ctx *ctx, const float *X, uint32_t n, const float *params, float *Y, int bf16)
{
	if(!ctx || !X || !n || !params || !Y) return GP_ERR_INVALID_ARG;
	MlpBufs b;
	gp_status st = mlp_bufs(ctx, n, b);
	if(st != GP_OK) return st;
	cudaStream_t s = ctx->stream;
	GP_CUDA(ctx, cudaMemcpyAsync(b.X, X, sizeof(float) * n * MLP_IN, cudaMemcpyHostToDevice, s));
	GP_CUDA(ctx, cudaMemcpyAsync(b.P, params, sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice, s));
	if(bf16) GP_CUDA(ctx, mlp_infer_bf16_device(b.P, b.X, (int) n, b.Y, s));
	else GP_CUDA(ctx, mlp_forward_f32_device(b.P, b.X, (int) n, b.work, b.Y, s));
	GP_CUDA(ctx, cudaMemcpyAsync(Y, b.Y, sizeof(float) * n * MLP_OUT, cudaMemcpyDeviceToHost, s));
	GP_CUDA(ctx, cudaStreamSynchronize(s));
	return GP_OK;
}

gp_status gp_normalize_ptp(gp_ctx *ctx, void *dist, gp_dtype dist_type, uint64_t n)
{
	if(!ctx || !dist) return GP_ERR_INVALID_ARG;
	if(!n) return GP_OK;
	const size_t sz = dist_type == GP_F64 ? 8 : 4;
	gp_status st = ensure_ws(ctx, n * sz + 256 + 64);
	if(st != GP_OK) return st;
	char *W = static_cast<char *>(ctx->ws);
	unsigned long long *tmp = reinterpret_cast<unsigned long long *>(W + align_up(n * sz, 256));
	cudaStream_t s = ctx->stream;
	GP_CUDA(ctx, cudaMemcpyAsync(W, dist, n * sz, cudaMemcpyHostToDevice, s));
	GP_CUDA(ctx, launch_normalize(W, dist_type == GP_F64, n, tmp, s));
	GP_CUDA(ctx, cudaMemcpyAsync(dist, W, n * sz, cudaMemcpyDeviceToHost, s));
	GP_CUDA(ctx, cudaStreamSynchronize(s));
	return GP_OK;
}

gp_status gp_fps(gp_ctx *ctx, gp_mesh *mesh, uint32_t *samples, uint32_t n_init, uint32_t cap, uint64_t n,
                 double radio, const gp_ptp_opts *opts, uint32_t *n_out, double *max_dist, double *seconds)
{
	if(!ctx || !mesh || !samples || !n_out || !max_dist || !n_init || n_init > cap) return GP_ERR_INVALID_ARG;
	for(uint32_t k = 0; k < n_init; k++)
		if(samples[k] >= mesh->nv) return GP_ERR_INVALID_ARG;
	// farthest_point_sampling_ptp_gpu (src/cuda/geodesics_ptp.cu:122-147)
	if(n >= mesh->nv) n = mesh->nv >> 1;
	n = n > n_init ? n - n_init : 0;  // the reference underflows when n < |samples|
	n = std::min<uint64_t>(n, cap - n_init);
	*n_out = n_init;
	*max_dist = INFINITY;
	if(seconds) *seconds = 0;
	if(!n) return GP_OK;
	const bool f64 = opts && opts->precision == GP_F64;
	// one call: layout and uploads once, then every sample's device work back
	// to back (sources, outputs and the argmax stay on the device); the
	// workspace is the context's, so nothing is allocated per call once it has
	// grown to this size
	FpsLoop loop{samples, n_init, (uint32_t) n, radio, n_init, (double) INFINITY};
	std::vector<char> scratch;  // the field's output is never read back
	Req r{mesh, samples, (uint32_t) (n_init + n), nullptr, 0, nullptr, nullptr, nullptr, nullptr};
	scratch.resize(1);
	r.dist = scratch.data();
	double sec = 0;
	const gp_status st = run(ctx, &r, 1, opts, f64 ? GP_F64 : GP_F32, false, false, Stage::ptp, nullptr, &sec, nullptr,
	                         nullptr, &loop);
	*n_out = loop.n_out;
	*max_dist = loop.max_dist;
	if(seconds) *seconds = sec;
	return st;
}

} // extern "C"
