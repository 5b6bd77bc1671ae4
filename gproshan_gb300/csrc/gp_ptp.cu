// PTP geodesics on the GPU: ring-renumbered layout, the persistent sweep
// launch with on-device convergence decisions, and the output passes.
//
// Reference path (gproshan): parallel_toplesets_propagation_gpu and
// run_ptp_gpu (src/cuda/geodesics_ptp.cu:20-85, 174-232), relax_ptp
// (:234-282), relative_error + thrust::count_if (:221-225, 284-299) and
// cu_update_step (:301-369).
//
// Layout.  Each field's vertices are renumbered by their position in `sorted`
// (the toplesets order), so every sweep window [limits[i], limits[j]) is one
// contiguous range and the check ring i is its head.  Unreached vertices all map
// to one sentinel id (distance INF), which reproduces the reference's view of
// them: they never enter a window and read as INF.
//
// Sweep.  One cooperative launch runs every sweep of every live field.  Each
// step, CTAs walk the tiles of all live windows (relax + the ring-i test);
// the last CTA to reach the grid barrier applies the reference's schedule
// rule to each field and lays out the next step's tiles.  No host round trip.
#include <cfloat>
#include <cmath>

#include "gp_common.cuh"

namespace gp {

namespace {

constexpr int NT = 512;  // threads of a grid-launch CTA (one tile = NT window vertices)

// Distance/label load: coherent (L2) when other CTAs of the launch write the
// buffer, plain otherwise.
template <class T, bool COH>
__device__ __forceinline__ T ld_d(const T *p)
{
	if constexpr(COH) return __ldcg(p);
	else return *p;
}

// ---------------------------------------------------------------------------
// FP32 planar update in closed form.
//
// With X0 = x0 - v, X1 = x1 - v, E = X1 - X0, e2 = |E|^2, A = |X0 x X1|
// (twice the triangle area) and dt = t1 - t0, the reference's quadratic
// (src/geodesics_ptp.cpp:220-236) has the root
//     p = t0 + (a1*dt + A*sqrt(e2 - dt^2)) / e2,   a1 = -X0.E,
// its discriminant is (e2 - dt^2) / det(q), and its upwind test
// c = Q (t - p) < 0 reads (X1.E)*delta + (X0.X1)*dt > 0 and
// a1*delta - |X0|^2*dt > 0 with delta = p - t0.  These are the same function
// as the reference's expression, written so that nothing large cancels: the
// Gram determinant is never formed and t enters only through dt.  Fallback,
// INF and degenerate-triangle behaviour follow the reference: INF inputs take
// the edge fallback, a degenerate triangle (A == 0) yields NaN and is ignored.
// ---------------------------------------------------------------------------
struct Nb32 {
	float x, y, z;  // X = P[u] - P[v]
	float t;        // old distance of u
	float q;        // |X|^2
	float l;        // |X|
	uint32_t u;
};

template <bool COH>
__device__ __forceinline__ Nb32 load_nb32(const float4 *__restrict__ P, const float *D, uint32_t u, float4 pv)
{
	Nb32 n;
	const float4 pu = __ldg(P + u);
	n.x = pu.x - pv.x;
	n.y = pu.y - pv.y;
	n.z = pu.z - pv.z;
	n.t = ld_d<float, COH>(D + u);
	n.q = fmaf(n.x, n.x, fmaf(n.y, n.y, n.z * n.z));
	n.l = sqrtf(n.q);
	n.u = u;
	return n;
}

__device__ __forceinline__ float update32(const Nb32 &a, const Nb32 &b)
{
	// fallback value dp[dp[1] < dp[0]]
	const float d0 = a.t + a.l, d1 = b.t + b.l;
	const float fb = d1 < d0 ? d1 : d0;
	if(a.t == INFINITY || b.t == INFINITY) return fb;
	const float ex = b.x - a.x, ey = b.y - a.y, ez = b.z - a.z;
	const float e2 = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
	const float cx = fmaf(a.y, b.z, -a.z * b.y);
	const float cy = fmaf(a.z, b.x, -a.x * b.z);
	const float cz = fmaf(a.x, b.y, -a.y * b.x);
	const float A = sqrtf(fmaf(cx, cx, fmaf(cy, cy, cz * cz)));
	if(!(A > 0.f)) return NAN;
	const float dt = b.t - a.t;
	const float r = fmaf(-dt, dt, e2);
	if(r < 0.f) return fb;
	const float a1 = -fmaf(a.x, ex, fmaf(a.y, ey, a.z * ez));
	const float a0 = fmaf(b.x, ex, fmaf(b.y, ey, b.z * ez));
	const float q01 = fmaf(a.x, b.x, fmaf(a.y, b.y, a.z * b.z));
	const float delta = fmaf(a1, dt, A * sqrtf(r)) / e2;
	if(fmaf(a0, delta, q01 * dt) > 0.f && fmaf(a1, delta, -a.q * dt) > 0.f)
		return a.t + delta;
	return fb;
}

// ---------------------------------------------------------------------------
// FP64 update: the reference formula (src/geodesics_ptp.cpp:201-262), term by
// term, with every product and sum rounded separately (no FMA contraction), so
// it matches the reference's compiled FP64 code bit for bit.
// ---------------------------------------------------------------------------
struct Nb64 {
	double x, y, z, t;
	uint32_t u;
};

__device__ __forceinline__ double dot64(double ax, double ay, double az, double bx, double by, double bz)
{
	return __dadd_rn(__dadd_rn(__dmul_rn(ax, bx), __dmul_rn(ay, by)), __dmul_rn(az, bz));
}

template <bool COH>
__device__ __forceinline__ Nb64 load_nb64(const double *__restrict__ Pd, const double *D, uint32_t u,
                                          double vx, double vy, double vz)
{
	Nb64 n;
	const double2 a = __ldg(reinterpret_cast<const double2 *>(Pd + 4 * (size_t) u));
	const double2 b = __ldg(reinterpret_cast<const double2 *>(Pd + 4 * (size_t) u) + 1);
	n.x = __dsub_rn(a.x, vx);
	n.y = __dsub_rn(a.y, vy);
	n.z = __dsub_rn(b.x, vz);
	n.t = ld_d<double, COH>(D + u);
	n.u = u;
	return n;
}

__device__ __forceinline__ double update64(const Nb64 &A0, const Nb64 &A1)
{
	const double X0x = A0.x, X0y = A0.y, X0z = A0.z, X1x = A1.x, X1y = A1.y, X1z = A1.z;
	const double t0 = A0.t, t1 = A1.t;
	const double q00 = dot64(X0x, X0y, X0z, X0x, X0y, X0z);
	const double q01 = dot64(X0x, X0y, X0z, X1x, X1y, X1z);
	const double q10 = dot64(X1x, X1y, X1z, X0x, X0y, X0z);
	const double q11 = dot64(X1x, X1y, X1z, X1x, X1y, X1z);
	const double det = __dsub_rn(__dmul_rn(q00, q11), __dmul_rn(q01, q10));
	const double Q00 = __ddiv_rn(q11, det);
	const double Q01 = __ddiv_rn(-q01, det);
	const double Q10 = __ddiv_rn(-q10, det);
	const double Q11 = __ddiv_rn(q00, det);
	const double delta = __dadd_rn(__dmul_rn(t0, __dadd_rn(Q00, Q10)), __dmul_rn(t1, __dadd_rn(Q01, Q11)));
	const double sQ = __dadd_rn(__dadd_rn(__dadd_rn(Q00, Q01), Q10), Q11);
	const double quad = __dsub_rn(
	    __dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(t0, t0), Q00), __dmul_rn(__dmul_rn(t0, t1), __dadd_rn(Q10, Q01))),
	              __dmul_rn(__dmul_rn(t1, t1), Q11)),
	    1.0);
	const double dis = __dsub_rn(__dmul_rn(delta, delta), __dmul_rn(sQ, quad));
	double p = __ddiv_rn(__dadd_rn(delta, __dsqrt_rn(dis)), sQ);
	const double tp0 = __dsub_rn(t0, p), tp1 = __dsub_rn(t1, p);
	const double nx = __dadd_rn(__dmul_rn(tp0, __dadd_rn(__dmul_rn(X0x, Q00), __dmul_rn(X1x, Q10))),
	                            __dmul_rn(tp1, __dadd_rn(__dmul_rn(X0x, Q01), __dmul_rn(X1x, Q11))));
	const double ny = __dadd_rn(__dmul_rn(tp0, __dadd_rn(__dmul_rn(X0y, Q00), __dmul_rn(X1y, Q10))),
	                            __dmul_rn(tp1, __dadd_rn(__dmul_rn(X0y, Q01), __dmul_rn(X1y, Q11))));
	const double nz = __dadd_rn(__dmul_rn(tp0, __dadd_rn(__dmul_rn(X0z, Q00), __dmul_rn(X1z, Q10))),
	                            __dmul_rn(tp1, __dadd_rn(__dmul_rn(X0z, Q01), __dmul_rn(X1z, Q11))));
	const double cond0 = dot64(X0x, X0y, X0z, nx, ny, nz);
	const double cond1 = dot64(X1x, X1y, X1z, nx, ny, nz);
	const double c0 = __dadd_rn(__dmul_rn(cond0, Q00), __dmul_rn(cond1, Q01));
	const double c1 = __dadd_rn(__dmul_rn(cond0, Q10), __dmul_rn(cond1, Q11));
	if(t0 == INFINITY || t1 == INFINITY || dis < 0 || c0 >= 0 || c1 >= 0)
	{
		const double dp0 = __dadd_rn(t0, __dsqrt_rn(q00));
		const double dp1 = __dadd_rn(t1, __dsqrt_rn(q11));
		p = dp1 < dp0 ? dp1 : dp0;
	}
	return p;
}

// ---------------------------------------------------------------------------
// Relaxation of one vertex: new = min(old[v], min over star triangles).
// ---------------------------------------------------------------------------
template <bool CL, bool COH>
__device__ __forceinline__ float relax32(const FieldDev &F, uint32_t v, const float *Do, const uint32_t *Co,
                                         uint32_t &lab)
{
	const uint32_t o0f = __ldg(F.off + v);
	const uint32_t o1 = __ldg(F.off + v + 1) & FAN_MASK;
	const uint32_t o0 = o0f & FAN_MASK;
	float best = ld_d<float, COH>(Do + v);
	if(CL) lab = ld_d<uint32_t, COH>(Co + v);
	if(o1 <= o0) return best;
	const float4 pv = __ldg(F.P + v);
	const uint32_t *fan = F.fan;
	const Nb32 first = load_nb32<COH>(F.P, Do, __ldg(fan + o0), pv);
	Nb32 prev = first;
	for(uint32_t e = o0 + 1; e < o1; e++)
	{
		const Nb32 cur = load_nb32<COH>(F.P, Do, __ldg(fan + e), pv);
		const float p = update32(prev, cur);
		if(p < best)
		{
			best = p;
			if(CL) lab = cur.t < prev.t ? ld_d<uint32_t, COH>(Co + cur.u) : ld_d<uint32_t, COH>(Co + prev.u);
		}
		prev = cur;
	}
	if(o0f & FAN_CLOSED)
	{
		const float p = update32(prev, first);
		if(p < best)
		{
			best = p;
			if(CL) lab = first.t < prev.t ? ld_d<uint32_t, COH>(Co + first.u) : ld_d<uint32_t, COH>(Co + prev.u);
		}
	}
	return best;
}

template <bool CL, bool COH>
__device__ __forceinline__ double relax64(const FieldDev &F, uint32_t v, const double *Do, const uint32_t *Co,
                                          uint32_t &lab)
{
	const uint32_t o0f = __ldg(F.off + v);
	const uint32_t o1 = __ldg(F.off + v + 1) & FAN_MASK;
	const uint32_t o0 = o0f & FAN_MASK;
	double best = ld_d<double, COH>(Do + v);
	if(CL) lab = ld_d<uint32_t, COH>(Co + v);
	if(o1 <= o0) return best;
	const double vx = F.Pd[4 * (size_t) v], vy = F.Pd[4 * (size_t) v + 1], vz = F.Pd[4 * (size_t) v + 2];
	const uint32_t *fan = F.fan;
	const Nb64 first = load_nb64<COH>(F.Pd, Do, __ldg(fan + o0), vx, vy, vz);
	Nb64 prev = first;
	for(uint32_t e = o0 + 1; e < o1; e++)
	{
		const Nb64 cur = load_nb64<COH>(F.Pd, Do, __ldg(fan + e), vx, vy, vz);
		const double p = update64(prev, cur);
		if(p < best)
		{
			best = p;
			if(CL) lab = cur.t < prev.t ? ld_d<uint32_t, COH>(Co + cur.u) : ld_d<uint32_t, COH>(Co + prev.u);
		}
		prev = cur;
	}
	if(o0f & FAN_CLOSED)
	{
		const double p = update64(prev, first);
		if(p < best)
		{
			best = p;
			if(CL) lab = first.t < prev.t ? ld_d<uint32_t, COH>(Co + first.u) : ld_d<uint32_t, COH>(Co + prev.u);
		}
	}
	return best;
}

struct PtpArgs {
	FieldDev *fields;
	FieldState *state;
	uint32_t n_fields;
	PlanDev *plan;
	GridSync *sync;
};

// Open the next sweep if the reference loop would run one
// (`while(i < j && iter++ < max_iter)` then the K/2 band,
// src/cuda/geodesics_ptp.cu:206-212), else retire the field.
__device__ __forceinline__ void open_sweep(const FieldDev &F, FieldState &st)
{
	if(st.i < st.j && st.iter < st.max_iter)
	{
		st.iter++;
		if(st.i < (st.j >> 1)) st.i = st.j >> 1;
		st.win_s = F.limits[st.i];
		st.win_e = F.limits[st.j];
		st.chk_e = F.limits[st.i + 1];
		st.live = 1;
		if(F.trace && st.n_iter < F.trace_cap)
		{
			F.trace[2 * st.n_iter] = st.i;
			F.trace[2 * st.n_iter + 1] = st.j;
		}
	}
	else st.live = 0;
}

// Relax window vertex v of field F (buffers d -> d^1) and, if v is in the
// check ring (v < chk_e), apply relative_error + is_ok
// (src/cuda/geodesics_ptp.cu:284-299, 371-375) in FP64.  Returns 1 if v fails
// the test.  COH: distances may have been written by other CTAs of this launch.
template <typename T, bool CL, bool COH>
__device__ __forceinline__ int sweep_vertex(const FieldDev &F, uint32_t d, uint32_t v, uint32_t chk_e)
{
	const T *Do = static_cast<const T *>(F.D[d]);
	T *Dn = static_cast<T *>(F.D[d ^ 1u]);
	const uint32_t *Co = CL ? F.C[d] : nullptr;
	uint32_t lab = 0;
	T nv;
	if constexpr(sizeof(T) == 4) nv = relax32<CL, COH>(F, v, reinterpret_cast<const float *>(Do), Co, lab);
	else nv = relax64<CL, COH>(F, v, reinterpret_cast<const double *>(Do), Co, lab);
	Dn[v] = nv;
	if(CL) F.C[d ^ 1u][v] = lab;
	if(v < chk_e)
	{
		const double o = (double) ld_d<T, COH>(Do + v);
		const double err = fabs((double) nv - o) / o;
		return !(err < F.tol);
	}
	return 0;
}

// ---------------------------------------------------------------------------
// classify: per field, the largest window its schedule can open
// (max over j of limits[j] - limits[j/2]) decides whether one CTA sweeps it
// (ptp_local_kernel) or the whole grid (ptp_kernel).  Also resets the
// schedule state so that fields with no sweep read back d = 0.
// ---------------------------------------------------------------------------
__global__ void classify_kernel(FieldDev *fields, FieldState *state, uint32_t n_fields, uint32_t local_window)
{
	const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
	if(warp >= n_fields) return;
	const FieldDev &F = fields[warp];
	FieldState &st = state[warp];
	const uint32_t nl = st.n_limits;
	uint32_t bound = 0;
	for(uint32_t j = 2 + lane; j < nl; j += 32) bound = max(bound, F.limits[j] - F.limits[j >> 1]);
	for(int o = 16; o; o >>= 1) bound = max(bound, __shfl_xor_sync(0xffffffffu, bound, o));
	if(lane == 0)
	{
		st.bound = bound;
		st.big = nl >= 3 && bound > local_window;
		st.nr = nl ? F.limits[nl - 1] : 0;
		st.i = 1;
		st.j = 2;
		st.d = 0;
		st.iter = 0;
		st.n_iter = 0;
		st.notok = 0;
		st.live = 0;
		st.relax = 0;
		st.max_iter = F.max_iter ? F.max_iter : (nl << 1);
	}
}

// ---------------------------------------------------------------------------
// One CTA sweeps one field from its first to its last sweep
// (run_ptp_gpu's loop, src/cuda/geodesics_ptp.cu:198-229): the window is
// swept in CTA-sized chunks, __syncthreads_or() both merges the ring-i test
// and separates the sweeps.  Every thread keeps the schedule in registers.
// ---------------------------------------------------------------------------
constexpr int LT = 512;

template <typename T, bool CL>
__global__ void __launch_bounds__(LT) ptp_local_kernel(FieldDev *fields, FieldState *state, uint32_t n_fields,
                                                       uint32_t *queue)
{
	__shared__ uint32_t s_f;
	for(;;)
	{
		if(threadIdx.x == 0) s_f = atomicAdd(queue, 1u);
		__syncthreads();
		const uint32_t f = s_f;
		__syncthreads();
		if(f >= n_fields) return;
		FieldState &gst = state[f];
		if(gst.big || gst.n_limits < 3) continue;
		const FieldDev &F = fields[f];
		FieldState st = {};
		st.i = 1;
		st.j = 2;
		st.max_iter = gst.max_iter;
		const uint32_t nl = gst.n_limits;
		open_sweep(F, st);
		while(st.live)
		{
			int bad = 0;
			for(uint32_t v = st.win_s + threadIdx.x; v < st.win_e; v += LT)
				bad |= sweep_vertex<T, CL, false>(F, st.d, v, st.chk_e);
			const int any = __syncthreads_or(bad);
			st.relax += st.win_e - st.win_s;
			if(!any) st.i++;
			if(st.j < nl - 1) st.j++;
			st.d ^= 1u;
			st.n_iter++;
			open_sweep(F, st);
		}
		if(threadIdx.x == 0)
		{
			gst.i = st.i;
			gst.j = st.j;
			gst.d = st.d;
			gst.iter = st.iter;
			gst.n_iter = st.n_iter;
			gst.relax = st.relax;
		}
	}
}

// ---------------------------------------------------------------------------
// Grid-wide persistent sweep of the big fields, all in lockstep: each step the
// CTAs walk the tiles of every live window, and the last CTA at the barrier
// applies the schedule rule to each field and lays out the next step.
// ---------------------------------------------------------------------------

// Tile plan of the next step, in the serial section (one CTA).
__device__ void ptp_plan(const PtpArgs &a)
{
	PlanDev *plan = a.plan;
	__shared__ uint32_t carry_f, carry_t;
	if(threadIdx.x == 0) { carry_f = 0; carry_t = 0; }
	__syncthreads();
	for(uint32_t base = 0; base < a.n_fields; base += NT)
	{
		const uint32_t f = base + threadIdx.x;
		uint32_t tiles = 0;
		if(f < a.n_fields && ldcg(&a.state[f].live))
			tiles = (ldcg(&a.state[f].win_e) - ldcg(&a.state[f].win_s) + NT - 1) / NT;
		const uint32_t is_act = tiles > 0;
		uint32_t tot_a, tot_t;
		const uint32_t ia = block_exclusive_scan<NT>(is_act, &tot_a);
		const uint32_t it = block_exclusive_scan<NT>(tiles, &tot_t);
		if(is_act)
		{
			plan->act[carry_f + ia] = f;
			plan->tile_start[carry_f + ia] = carry_t + it;
		}
		__syncthreads();
		if(threadIdx.x == 0) { carry_f += tot_a; carry_t += tot_t; }
		__syncthreads();
	}
	if(threadIdx.x == 0)
	{
		plan->n_act = carry_f;
		plan->total_tiles = carry_t;
		plan->tile_start[carry_f] = carry_t;
		plan->live = carry_f > 0;
		plan->step++;
	}
	__syncthreads();
}

// First serial section: open the first sweep of every big field.
__device__ void ptp_start(const PtpArgs &a)
{
	for(uint32_t f = threadIdx.x; f < a.n_fields; f += NT)
	{
		FieldState &st = a.state[f];
		if(!st.big) continue;
		open_sweep(a.fields[f], st);
	}
	if(threadIdx.x == 0) a.plan->step = 0;
	__syncthreads();
	ptp_plan(a);
}

// Serial section after a sweep: the reference's schedule update
// (src/cuda/geodesics_ptp.cu:224-228), then the next sweep's window.
__device__ void ptp_advance(const PtpArgs &a)
{
	const uint32_t n_act = ldcg(&a.plan->n_act);
	for(uint32_t ai = threadIdx.x; ai < n_act; ai += NT)
	{
		const uint32_t f = ldcg(a.plan->act + ai);
		const FieldDev &F = a.fields[f];
		FieldState *g = a.state + f;
		// private copy: every field is owned by one thread of the serial CTA
		FieldState st = {};
		st.i = ldcg(&g->i);
		st.j = ldcg(&g->j);
		st.d = ldcg(&g->d);
		st.iter = ldcg(&g->iter);
		st.max_iter = ldcg(&g->max_iter);
		st.n_iter = ldcg(&g->n_iter);
		st.win_s = ldcg(&g->win_s);
		st.win_e = ldcg(&g->win_e);
		st.relax = ldcg(&g->relax);
		const uint32_t nl = ldcg(&g->n_limits);
		st.relax += st.win_e - st.win_s;
		if(!ldcg(&g->notok)) st.i++;
		if(st.j < nl - 1) st.j++;
		st.d ^= 1u;
		st.n_iter++;
		open_sweep(F, st);
		g->i = st.i;
		g->j = st.j;
		g->d = st.d;
		g->iter = st.iter;
		g->n_iter = st.n_iter;
		g->relax = st.relax;
		g->notok = 0;
		g->live = st.live;
		g->win_s = st.win_s;
		g->win_e = st.win_e;
		g->chk_e = st.chk_e;
	}
	__syncthreads();
	ptp_plan(a);
}

template <typename T, bool CL>
__global__ void __launch_bounds__(NT) ptp_kernel(PtpArgs a)
{
	uint32_t gen = 0;
	if(!grid_sync(a.sync, gen, [&] { ptp_start(a); })) return;
	const uint32_t lane = threadIdx.x & 31;

	for(;;)
	{
		if(!ld_relaxed(&a.plan->live) || ld_relaxed(&a.sync->abort)) break;
		const uint32_t T_tiles = ldcg(&a.plan->total_tiles);
		const uint32_t n_act = ldcg(&a.plan->n_act);
		for(uint32_t k = blockIdx.x; k < T_tiles; k += gridDim.x)
		{
			const uint32_t ai = upper_index<true>(a.plan->tile_start, n_act, k);
			const uint32_t f = ldcg(a.plan->act + ai);
			const FieldDev &F = a.fields[f];
			const FieldState *stp = a.state + f;
			const uint32_t d = ldcg(&stp->d);
			const uint32_t win_e = ldcg(&stp->win_e), chk_e = ldcg(&stp->chk_e);
			const uint32_t v = ldcg(&stp->win_s) + (k - ldcg(a.plan->tile_start + ai)) * NT + threadIdx.x;
			int bad = 0;
			if(v < win_e) bad = sweep_vertex<T, CL, true>(F, d, v, chk_e);
			// one atomic per warp that saw a failure, no block barrier per tile
			if(__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(&a.state[f].notok, 1u);
		}
		if(!grid_sync(a.sync, gen, [&] { ptp_advance(a); })) return;
	}
}

// ---------------------------------------------------------------------------
// Renumbering passes over the concatenated per-field slots
// (slot f = [base[f], base[f+1]), slot size nv + ns + 2).
// ---------------------------------------------------------------------------
struct CatArgs {
	FieldDev *fields;
	FieldState *state;
	const uint32_t *base;  // F + 1
	uint32_t n_fields;
	uint32_t total;
	uint32_t *cnt;         // total (+1) counts, then global fan offsets after the scan
};

__global__ void inv_clear_kernel(CatArgs c)
{
	for(uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < c.total; g += gridDim.x * blockDim.x)
	{
		const uint32_t f = upper_index(c.base, c.n_fields, g);
		const uint32_t k = g - c.base[f];
		if(k < c.fields[f].m.nv) c.fields[f].inv[k] = 0;
	}
}

__global__ void inv_set_kernel(CatArgs c)
{
	for(uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < c.total; g += gridDim.x * blockDim.x)
	{
		const uint32_t f = upper_index(c.base, c.n_fields, g);
		const uint32_t k = g - c.base[f];
		const FieldState &st = c.state[f];
		const uint32_t nr = st.n_limits ? c.fields[f].limits[st.n_limits - 1] : 0;
		if(k < nr) atomicMax(&c.fields[f].inv[c.fields[f].sorted[k]], k + 1);
	}
}

__global__ void count_kernel(CatArgs c)
{
	for(uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < c.total; g += gridDim.x * blockDim.x)
	{
		const uint32_t f = upper_index(c.base, c.n_fields, g);
		const uint32_t k = g - c.base[f];
		const FieldDev &F = c.fields[f];
		const FieldState &st = c.state[f];
		const uint32_t nr = st.n_limits ? F.limits[st.n_limits - 1] : 0;
		uint32_t n = 0;
		if(k < nr)
		{
			const uint32_t v = F.sorted[k];
			n = (F.m.fan_off[v + 1] & FAN_MASK) - (F.m.fan_off[v] & FAN_MASK);
		}
		c.cnt[g] = n;
	}
}

template <typename T, bool CL>
__global__ void fill_kernel(CatArgs c)
{
	for(uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < c.total; g += gridDim.x * blockDim.x)
	{
		const uint32_t f = upper_index(c.base, c.n_fields, g);
		const uint32_t k = g - c.base[f];
		const FieldDev &F = c.fields[f];
		const FieldState &st = c.state[f];
		const uint32_t nr = st.n_limits ? F.limits[st.n_limits - 1] : 0;
		const uint32_t n0 = st.n_limits >= 2 ? F.limits[1] : nr;
		T *D0 = static_cast<T *>(F.D[0]);
		T *D1 = static_cast<T *>(F.D[1]);
		if(k < nr)
		{
			const uint32_t v = F.sorted[k];
			const uint32_t o0f = F.m.fan_off[v];
			const uint32_t o0 = o0f & FAN_MASK, o1 = F.m.fan_off[v + 1] & FAN_MASK;
			const uint32_t dst = c.cnt[g];
			for(uint32_t e = o0; e < o1; e++)
			{
				const uint32_t u = F.m.fan[e];
				const uint32_t iu = F.inv[u];
				F.fan[dst + (e - o0)] = iu ? iu - 1 : nr;
			}
			F.off[k] = dst | (o0f & FAN_CLOSED);
			F.P[k] = F.m.pos[v];
			if(F.Pd)
			{
				F.Pd[4 * (size_t) k] = F.m.posd[4 * (size_t) v];
				F.Pd[4 * (size_t) k + 1] = F.m.posd[4 * (size_t) v + 1];
				F.Pd[4 * (size_t) k + 2] = F.m.posd[4 * (size_t) v + 2];
				F.Pd[4 * (size_t) k + 3] = 0.0;
			}
			const T d0 = k < n0 ? T(0) : T(INFINITY);
			D0[k] = d0;
			D1[k] = d0;
			if(CL)
			{
				// sources carry the 1-based index of their last occurrence
				// (src/cuda/geodesics_ptp.cu:191-192); others the caller's label
				uint32_t lab = F.clusters_in ? F.clusters_in[v] : 0u;
				if(k < n0) lab = F.inv[v];
				F.C[0][k] = lab;
				F.C[1][k] = lab;
			}
		}
		else if(k == nr)
		{
			F.off[k] = c.cnt[g];
			F.P[k] = make_float4(0.f, 0.f, 0.f, 0.f);
			if(F.Pd)
				for(int q = 0; q < 4; q++) F.Pd[4 * (size_t) k + q] = 0.0;
			D0[k] = T(INFINITY);
			D1[k] = T(INFINITY);
			if(CL) { F.C[0][k] = 0; F.C[1][k] = 0; }
		}
	}
}

template <typename T, bool CL>
__global__ void gather_kernel(CatArgs c)
{
	for(uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < c.total; g += gridDim.x * blockDim.x)
	{
		const uint32_t f = upper_index(c.base, c.n_fields, g);
		const uint32_t v = g - c.base[f];
		const FieldDev &F = c.fields[f];
		if(v >= F.m.nv) continue;
		const FieldState &st = c.state[f];
		const uint32_t iv = F.inv[v];
		const uint32_t k = iv ? iv - 1 : st.nr;
		const T x = static_cast<const T *>(F.D[st.d])[k];
		if(F.out_f64) static_cast<double *>(F.dist_out)[v] = (double) x;
		else static_cast<float *>(F.dist_out)[v] = (float) x;
		if(CL && F.clusters_out)
			F.clusters_out[v] = iv ? F.C[st.d][k] : (F.clusters_in ? F.clusters_in[v] : 0u);
	}
}

// ---------------------------------------------------------------------------
// normalize_ptp and argmax |x|
// ---------------------------------------------------------------------------
template <typename T>
__global__ void max_finite_kernel(const T *x, uint64_t n, unsigned long long *out)
{
	unsigned long long m = 0;
	for(uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x)
	{
		const double v = (double) x[i];
		if(v < INFINITY && v > 0) m = max(m, (unsigned long long) __double_as_longlong(v));
	}
	for(int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
	if((threadIdx.x & 31) == 0) atomicMax(out, m);
}

template <typename T>
__global__ void divide_kernel(T *x, uint64_t n, const unsigned long long *mx)
{
	const T m = (T) __longlong_as_double((long long) *mx);
	for(uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x)
		x[i] /= m;
}

template <typename T>
__global__ void max_abs_kernel(const T *x, uint32_t n, unsigned long long *out)
{
	unsigned long long m = 0;
	for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
		m = max(m, (unsigned long long) __double_as_longlong(fabs((double) x[i])));
	for(int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
	if((threadIdx.x & 31) == 0) atomicMax(out, m);
}

template <typename T>
__global__ void first_index_kernel(const T *x, uint32_t n, unsigned long long *out)
{
	const unsigned long long m = out[0];
	unsigned long long best = ~0ull;
	for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
		if((unsigned long long) __double_as_longlong(fabs((double) x[i])) == m) { best = i; break; }
	for(int o = 16; o; o >>= 1) best = min(best, __shfl_xor_sync(0xffffffffu, best, o));
	if((threadIdx.x & 31) == 0 && best != ~0ull) atomicMin(out + 1, best);
}

unsigned grid_for(uint64_t n)
{
	return (unsigned) std::max<uint64_t>(1, std::min<uint64_t>((n + 255) / 256, 152ull * 32));
}

} // namespace

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------

cudaError_t launch_renumber_batch(FieldDev *fields, FieldState *state, const uint32_t *base, uint32_t n_fields,
                                  uint32_t total, uint32_t *cnt, uint32_t *scan_tmp, bool f64, bool clusters,
                                  cudaStream_t s)
{
	CatArgs c{fields, state, base, n_fields, total, cnt};
	const unsigned nb = grid_for(total);
	inv_clear_kernel<<<nb, 256, 0, s>>>(c);
	inv_set_kernel<<<nb, 256, 0, s>>>(c);
	count_kernel<<<nb, 256, 0, s>>>(c);
	cudaError_t e = launch_scan_u32(cnt, cnt, total, scan_tmp, s);
	if(e != cudaSuccess) return e;
	if(f64)
	{
		if(clusters) fill_kernel<double, true><<<nb, 256, 0, s>>>(c);
		else fill_kernel<double, false><<<nb, 256, 0, s>>>(c);
	}
	else
	{
		if(clusters) fill_kernel<float, true><<<nb, 256, 0, s>>>(c);
		else fill_kernel<float, false><<<nb, 256, 0, s>>>(c);
	}
	return cudaGetLastError();
}

cudaError_t launch_gather_batch(FieldDev *fields, FieldState *state, const uint32_t *base, uint32_t n_fields,
                                uint32_t total, bool f64, bool clusters, cudaStream_t s)
{
	CatArgs c{fields, state, base, n_fields, total, nullptr};
	const unsigned nb = grid_for(total);
	if(f64)
	{
		if(clusters) gather_kernel<double, true><<<nb, 256, 0, s>>>(c);
		else gather_kernel<double, false><<<nb, 256, 0, s>>>(c);
	}
	else
	{
		if(clusters) gather_kernel<float, true><<<nb, 256, 0, s>>>(c);
		else gather_kernel<float, false><<<nb, 256, 0, s>>>(c);
	}
	return cudaGetLastError();
}

static const void *ptp_kernel_ptr(bool f64, bool clusters)
{
	if(f64) return clusters ? (const void *) ptp_kernel<double, true> : (const void *) ptp_kernel<double, false>;
	return clusters ? (const void *) ptp_kernel<float, true> : (const void *) ptp_kernel<float, false>;
}

int ptp_max_ctas(int device, bool f64, bool clusters)
{
	int nsm = 0, per = 0;
	cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, ptp_kernel_ptr(f64, clusters), NT, 0);
	return nsm * per;
}

int ptp_threads() { return NT; }

static const void *ptp_local_ptr(bool f64, bool clusters)
{
	if(f64)
		return clusters ? (const void *) ptp_local_kernel<double, true> : (const void *) ptp_local_kernel<double, false>;
	return clusters ? (const void *) ptp_local_kernel<float, true> : (const void *) ptp_local_kernel<float, false>;
}

int ptp_local_max_ctas(int device, bool f64, bool clusters)
{
	int nsm = 0, per = 0;
	cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, ptp_local_ptr(f64, clusters), LT, 0);
	return nsm * per;
}

cudaError_t launch_classify(FieldDev *fields, FieldState *state, uint32_t n_fields, uint32_t local_window,
                            cudaStream_t s)
{
	if(!n_fields) return cudaSuccess;
	classify_kernel<<<(n_fields * 32 + 255) / 256, 256, 0, s>>>(fields, state, n_fields, local_window);
	return cudaGetLastError();
}

// queue: one word, zeroed here (the field ticket)
cudaError_t launch_ptp_local(FieldDev *fields, FieldState *state, uint32_t n_fields, uint32_t *queue,
                             uint32_t ctas, bool f64, bool clusters, cudaStream_t s)
{
	cudaError_t e = cudaMemsetAsync(queue, 0, sizeof(uint32_t), s);
	if(e != cudaSuccess) return e;
	ctas = std::max<uint32_t>(1, std::min<uint32_t>(ctas, n_fields));
	void *args[] = {&fields, &state, &n_fields, &queue};
	return cudaLaunchKernel(ptp_local_ptr(f64, clusters), dim3(ctas), dim3(LT), args, 0, s);
}

cudaError_t launch_ptp(FieldDev *fields, FieldState *state, uint32_t n_fields, PlanDev *plan, GridSync *sync,
                       uint32_t ctas, bool f64, bool clusters, cudaStream_t s)
{
	PtpArgs a{fields, state, n_fields, plan, sync};
	void *args[] = {&a};
	cudaError_t e = cudaMemsetAsync(sync, 0, sizeof(GridSync), s);
	if(e != cudaSuccess) return e;
	return cudaLaunchCooperativeKernel(ptp_kernel_ptr(f64, clusters), dim3(ctas), dim3(NT), args, 0, s);
}

cudaError_t launch_normalize(void *dist, bool f64, uint64_t n, unsigned long long *tmp, cudaStream_t s)
{
	cudaError_t e = cudaMemsetAsync(tmp, 0, sizeof(unsigned long long), s);
	if(e != cudaSuccess) return e;
	const unsigned nb = grid_for(n);
	if(f64)
	{
		max_finite_kernel<double><<<nb, 256, 0, s>>>((const double *) dist, n, tmp);
		divide_kernel<double><<<nb, 256, 0, s>>>((double *) dist, n, tmp);
	}
	else
	{
		max_finite_kernel<float><<<nb, 256, 0, s>>>((const float *) dist, n, tmp);
		divide_kernel<float><<<nb, 256, 0, s>>>((float *) dist, n, tmp);
	}
	return cudaGetLastError();
}

// out[0] = bits of max |x|, out[1] = first index holding it (cublasI?amax, 0-based)
cudaError_t launch_argmax_abs(const void *dist, bool f64, uint32_t n, unsigned long long *out, cudaStream_t s)
{
	unsigned long long init[2] = {0ull, ~0ull};
	cudaError_t e = cudaMemcpyAsync(out, init, sizeof(init), cudaMemcpyHostToDevice, s);
	if(e != cudaSuccess) return e;
	const unsigned nb = grid_for(n);
	if(f64)
	{
		max_abs_kernel<double><<<nb, 256, 0, s>>>((const double *) dist, n, out);
		first_index_kernel<double><<<nb, 256, 0, s>>>((const double *) dist, n, out);
	}
	else
	{
		max_abs_kernel<float><<<nb, 256, 0, s>>>((const float *) dist, n, out);
		first_index_kernel<float><<<nb, 256, 0, s>>>((const float *) dist, n, out);
	}
	return cudaGetLastError();
}

} // namespace gp
