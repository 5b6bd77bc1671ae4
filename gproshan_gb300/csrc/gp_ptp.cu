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
// Sweeps.  Every field starts on one CTA (ptp_local_kernel), which runs its
// sweeps with CTA barriers as long as the windows stay small; a field whose
// window outgrows local_window is handed, mid-schedule, to the grid-wide
// launch: ptp_kernel (lockstep: one sweep of every live field per step, a
// counting grid barrier, every CTA applying the reference's schedule rule to
// its own copy of the schedules) or ptp_queue_kernel (work queue: per-field
// claims and completions, no grid barrier).  No host round trip.
#include <cfloat>
#include <cmath>
#include <type_traits>

#include "gp_bfs.cuh"
#include "gp_common.cuh"
#include "gp_mlp.h"

namespace gp {

namespace {

// Launch shape of the grid-wide sweeps, fixed at compile time (a -D override
// builds a variant for measurement): NT threads per CTA, GRID_MINB CTAs per
// SM.  One 1024-thread CTA per SM measured fastest on the benchmark batch
// (768 and 512 threads: 6 % and 34 % slower).
#ifndef GP_NT
#define GP_NT 1024
#endif
#ifndef GP_GRID_MINB
#define GP_GRID_MINB 1
#endif
constexpr int NT = GP_NT;  // threads of a grid-launch CTA

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
	float t;        // old distance of u, relative to the vertex's base (rounded)
	float te;       // rounding residual of t: t + te is the relative distance to ~1e-14 of an edge
	float q;        // |X|^2
	float l;        // |X|
	uint32_t u;
};

// Knuth's TwoSum: s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
	s = a + b;
	const float bb = s - a;
	e = (a - (s - bb)) + (b - bb);
}

// sqrt and reciprocal to about 1 ulp on the SFU (PTX .approx forms).  Used on
// edge-sized offsets only; correctly rounded forms give no measurable change
// in the results (the error budget is set by the sums below, not by these).
__device__ __forceinline__ float sqrt_a(float x)
{
	float y;
	asm("sqrt.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
	return y;
}

__device__ __forceinline__ float rcp_a(float x)
{
	float y;
	asm("rcp.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
	return y;
}

// A triangle's candidate: p = t + x rounded (what the minimum is taken on),
// with the operands kept so that the winner's value can be formed exactly:
// (t + te) + x.  Rounding every candidate to a float and carrying that into
// the next sweep biases the minimum low by a fraction of an ulp per update;
// on meshes with long needle triangles (edge ratios ~20:1) the ill-conditioned
// updates then amplify it to ~1e-4 of the distance.  Forming the winner
// exactly keeps the FP32 path within ~2e-7 of the FP64 reference there.
struct Cand32 {
	float p, t, x, te;
};

__device__ __forceinline__ Cand32 update32(const Nb32 &a, const Nb32 &b)
{
	// fallback value dp[dp[1] < dp[0]]
	const float d0 = a.t + a.l, d1 = b.t + b.l;
	const bool fb1 = d1 < d0;
	const float fb = fb1 ? d1 : d0;
	const float ft = fb1 ? b.t : a.t, fx = fb1 ? b.l : a.l, fe = fb1 ? b.te : a.te;
	// every lane evaluates the whole update and the cases are selected at the
	// end (no divergence inside a warp)
	const float ex = b.x - a.x, ey = b.y - a.y, ez = b.z - a.z;
	const float e2 = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
	const float cx = fmaf(a.y, b.z, -a.z * b.y);
	const float cy = fmaf(a.z, b.x, -a.x * b.z);
	const float cz = fmaf(a.x, b.y, -a.y * b.x);
	const float A2 = fmaf(cx, cx, fmaf(cy, cy, cz * cz));
	const float dt = (b.t - a.t) + (b.te - a.te);
	const float r = fmaf(-dt, dt, e2);
	const float a1 = -fmaf(a.x, ex, fmaf(a.y, ey, a.z * ez));
	const float a0 = fmaf(b.x, ex, fmaf(b.y, ey, b.z * ez));
	const float q01 = fmaf(a.x, b.x, fmaf(a.y, b.y, a.z * b.z));
	// A*sqrt(r) = sqrt(A^2 r): one root per triangle
	const float delta = fmaf(a1, dt, sqrt_a(A2 * fmaxf(r, 0.f))) * rcp_a(e2);
	const bool planar = fmaf(a0, delta, q01 * dt) > 0.f && fmaf(a1, delta, -a.q * dt) > 0.f && !(r < 0.f);
	Cand32 c;
	c.p = planar ? a.t + delta : fb;
	c.t = planar ? a.t : ft;
	c.x = planar ? delta : fx;
	c.te = planar ? a.te : fe;
	// An INF input never passes the planar test (dt is +-INF, so r = -INF;
	// or both INF, dt and the test are NaN), so the candidate is already the
	// edge fallback then.  A degenerate triangle (A == 0) yields NaN and is
	// ignored, except with an INF input: the reference checks INF first.
	if(!(A2 > 0.f) && fmaxf(a.t, b.t) != INFINITY) c.p = NAN;
	return c;
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
	// q10 = X1.X0 equals q01 bit for bit (IEEE products commute and the sums
	// run in the same order), hence Q10 == Q01: one division fewer
	const double q10 = q01;
	const double q11 = dot64(X1x, X1y, X1z, X1x, X1y, X1z);
	const double det = __dsub_rn(__dmul_rn(q00, q11), __dmul_rn(q01, q10));
	const double Q00 = __ddiv_rn(q11, det);
	const double Q01 = __ddiv_rn(-q01, det);
	const double Q10 = Q01;
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
// Fan entries whose loads are issued together before any update is computed:
// a vertex of valence <= FB costs three dependent memory trips (offset, fan
// indices, neighbour positions + distances) instead of two per neighbour.
constexpr uint32_t FB = 8;

template <bool CL, bool COH>
__device__ __forceinline__ void take32(const Nb32 &a, const Nb32 &b, Cand32 &best, uint32_t &lab, const uint32_t *Co)
{
	// Every triangle is solved: a skip test on min(t0, t1) >= best costs more
	// issue slots than the solves it saves (the update is branch-free).
	const Cand32 c = update32(a, b);
	if(c.p < best.p)
	{
		best = c;
		// GPU label rule (src/cuda/geodesics_ptp.cu:277): a = x0 (next), b = x1
		// (prev); the old distances compared exactly, as (t, te) pairs
		if(CL)
		{
			const bool pb = b.t < a.t || (b.t == a.t && b.te < a.te);
			lab = pb ? ld_d<uint32_t, COH>(Co + b.u) : ld_d<uint32_t, COH>(Co + a.u);
		}
	}
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

// Open the next sweep if the reference loop would run one
// (`while(i < j && iter++ < max_iter)` then the K/2 band,
// src/cuda/geodesics_ptp.cu:206-212), else retire the field.
__device__ __forceinline__ void open_sweep(const FieldDev &F, FieldState &st, bool trace)
{
	if(st.i < st.j && st.iter < st.max_iter)
	{
		st.iter++;
		if(st.i < (st.j >> 1)) st.i = st.j >> 1;
		st.win_s = ldcg(F.limits + st.i);
		st.win_e = ldcg(F.limits + st.j);
		st.chk_e = ldcg(F.limits + st.i + 1);
		st.live = 1;
		if(trace && F.trace && st.n_iter < F.trace_cap)
		{
			F.trace[2 * st.n_iter] = st.i;
			F.trace[2 * st.n_iter + 1] = st.j;
		}
	}
	else st.live = 0;
}

// The schedule rule applied after every sweep (src/cuda/geodesics_ptp.cu:224-228).
__device__ __forceinline__ void close_sweep(FieldState &st, bool converged)
{
	st.relax += st.win_e - st.win_s;
	if(converged) st.i++;
	if(st.j < st.n_limits - 1) st.j++;
	st.d ^= 1u;
	st.n_iter++;
}

// ---------------------------------------------------------------------------
// FP32 path storage: distances are double-float pairs (hi, lo).  A vertex is
// relaxed on distances RELATIVE to a base (its own distance, or while it is
// still INF its smallest loaded neighbour's), so the FP32 solver only sees
// edge-sized offsets and rounds to ~1e-7 of an edge instead of ~1e-7 of the
// distance; the new value is base + best offset, formed exactly in
// double-float.  This keeps the ring-i test (relative change < tol) on the
// same side of the threshold as an FP64 run, sweep after sweep.
// ---------------------------------------------------------------------------
template <bool COH>
__device__ __forceinline__ float2 ld2(const float2 *p)
{
	if constexpr(COH) return __ldcg(p);
	else return *p;
}

// Change flag: distances are >= 0, so the sign bit of a stored hi word is free
// and marks a value that differs (bitwise) from the one the same sweep read.
// Buffers start with the flag set on every vertex but the sources (a vertex
// never relaxed counts as changed).  A window vertex whose own value and every
// neighbour's value are unflagged, with no neighbour below the window, was
// relaxed in the previous sweep on exactly the inputs it would read now: its
// new value is the value it holds, and the solves are skipped (the value is
// stored again, unflagged).  The neighbours below the window are excluded
// because they are no longer rewritten, so their two buffers can differ while
// their flags are stale.  The flags cost one more memory trip, so they are
// read only by warps whose own 32 values are all unflagged, and only in steps
// with at least one tile per warp of the launch: a lighter step is bound by
// the latency of its slowest tile, and the skip would only lengthen it.
__device__ __forceinline__ float2 unflag(float2 d) { return make_float2(fabsf(d.x), d.y); }
__device__ __forceinline__ bool flagged(float h) { return (__float_as_uint(h) >> 31) != 0u; }

// (t, residual): t = (dv - base) rounded, t + residual the exact difference
// up to the lo parts' own rounding.  The hi difference is formed exactly too
// (TwoSum): a neighbour much nearer or farther than the base (a long edge next
// to a short one) is not within Sterbenz range, and dropping that rounding
// biases the FP32 solver low by ~1e-5 of the distance on anisotropic meshes.
__device__ __forceinline__ float2 rel_to(float2 dv, float bh, float bl)
{
	if(dv.x == INFINITY) return make_float2(INFINITY, 0.f);
	float h, eh;
	two_sum(dv.x, -bh, h, eh);
	const float l = (dv.y - bl) + eh;
	const float t = h + l;
	return make_float2(t, l - (t - h));
}

__device__ __forceinline__ Nb32 make_nb(float4 pu, float2 t, float4 pv, uint32_t u)
{
	Nb32 n;
	n.x = pu.x - pv.x;
	n.y = pu.y - pv.y;
	n.z = pu.z - pv.z;
	n.t = t.x;
	n.te = t.y;
	n.q = fmaf(n.x, n.x, fmaf(n.y, n.y, n.z * n.z));
	n.l = sqrt_a(n.q);
	n.u = u;
	return n;
}

__device__ __forceinline__ Nb32 make_nb_lean(float4 pu, float2 t, float4 pv)
{
	Nb32 n;
	n.x = pu.x - pv.x;
	n.y = pu.y - pv.y;
	n.z = pu.z - pv.z;
	n.t = t.x;
	n.te = t.y;
	n.q = fmaf(n.x, n.x, fmaf(n.y, n.y, n.z * n.z));
	n.l = sqrt_a(n.q);
	n.u = 0;
	return n;
}

// Relaxation of one vertex on the FP32 path: new = min(old, star updates),
// with the strict `if(p < best)` order of the reference (relax_ptp,
// src/cuda/geodesics_ptp.cu:234-282).  All fan indices of a vertex of valence
// <= FB are fetched at once, the neighbours in chunks of FC (bounded
// registers, several loads in flight).  Returns the new (hi, lo) pair.
#ifndef GP_FC
#define GP_FC 2
#endif
// Unlabelled FP32 sweeps take relax32_lean (1) or the triangle-by-triangle
// relax32 (0, a measurement build).
#ifndef GP_LEAN
#define GP_LEAN 1
#endif
constexpr uint32_t FC = GP_FC;

// (bh, bl) + x, exactly in double-float
// The new distance base + (t + te + x), formed exactly in double-float from
// the winning candidate's operands.
__device__ __forceinline__ float2 df_result(float bh, float bl, const Cand32 &c)
{
	float s, e;
	two_sum(c.t, c.x, s, e);
	float h0, e0;
	two_sum(bh, s, h0, e0);
	e0 += (bl + c.te) + e;
	const float h = h0 + e0;
	return make_float2(h, e0 - (h - h0));
}

// Vertices of valence above 8: the fan from the CSR lists, one neighbour at a time.
template <bool CL, bool COH>
__device__ __noinline__ float2 relax32_csr(const FieldDev &F, uint32_t v, const float2 *Do, const uint32_t *Co,
                                           uint32_t &lab, float2 vd, float4 pv)
{
	const uint32_t o0f = __ldg(F.off + v);
	const uint32_t o1 = __ldg(F.off + v + 1) & FAN_MASK;
	const uint32_t o0 = o0f & FAN_MASK;
	const uint32_t n = o1 > o0 ? o1 - o0 : 0u;
	if(!n) return vd;
	const uint32_t *fan = F.fan + o0;
	float bh = vd.x, bl = vd.y;
	if(bh == INFINITY)
	{
		float m = INFINITY;
		for(uint32_t k = 0; k < n; k++) m = fminf(m, fabsf(ld2<COH>(Do + __ldg(fan + k)).x));
		bh = m == INFINITY ? 0.f : m;
		bl = 0.f;
	}
	const float old_rel = vd.x == INFINITY ? INFINITY : 0.f;
	Cand32 best = {old_rel, 0.f, 0.f, 0.f};
	const uint32_t w0 = __ldg(fan);
	const Nb32 first = make_nb(__ldg(F.P + w0), rel_to(unflag(ld2<COH>(Do + w0)), bh, bl), pv, w0);
	Nb32 last = first;
	for(uint32_t e = 1; e < n; e++)
	{
		const uint32_t w = __ldg(fan + e);
		const Nb32 cur = make_nb(__ldg(F.P + w), rel_to(unflag(ld2<COH>(Do + w)), bh, bl), pv, w);
		take32<CL, COH>(last, cur, best, lab, Co);
		last = cur;
	}
	if(o0f & FAN_CLOSED) take32<CL, COH>(last, first, best, lab, Co);
	if(!(best.p < old_rel)) return vd;
	return df_result(bh, bl, best);
}

template <bool CL, bool COH>
__device__ __forceinline__ float2 relax32(const FieldDev &F, uint32_t v, const float2 *Do, const uint32_t *Co,
                                          uint32_t &lab, uint32_t win_s, bool try_skip, float2 &vd, bool &skip)
{
	// the fan row, the vertex's own distance and position: one memory trip
	const uint4 ra = __ldg(F.fan8 + 2 * (size_t) v), rb = __ldg(F.fan8 + 2 * (size_t) v + 1);
	const float2 vs = ld2<COH>(Do + v);
	vd = unflag(vs);
	const float4 pv = __ldg(F.P + v);
	if(CL) lab = ld_d<uint32_t, COH>(Co + v);
	uint32_t u[FB] = {ra.x & FAN8_ID_MASK, ra.y, ra.z, ra.w, rb.x, rb.y, rb.z, rb.w};
	const bool closed = (ra.x & FAN_CLOSED) != 0;
	if(rb.w == FAN8_OVERFLOW) return relax32_csr<CL, COH>(F, v, Do, Co, lab, vd, pv);
	const uint32_t n = (ra.x >> FAN8_N_SHIFT) & 15u;
	if(!n) return vd;
	// inputs unchanged since the previous sweep: the value stands (labels
	// always take the full path: a tie can move a label without a distance)
	if(!CL && try_skip)
	{
		const unsigned am = __activemask();
		if(__all_sync(am, !flagged(vs.x)))
		{
			bool same = true;
#pragma unroll
			for(uint32_t k = 0; k < FB; k++)
				if(k < n) same &= u[k] >= win_s && !flagged(ld_d<float, COH>(reinterpret_cast<const float *>(Do + u[k])));
			if(same)
			{
				skip = true;
				return vd;
			}
		}
	}
	// base of the relative distances: the vertex itself, or (while it is INF)
	// its smallest neighbour
	float bh = vd.x, bl = vd.y;
	if(bh == INFINITY)
	{
		float m = INFINITY;
#pragma unroll
		for(uint32_t k = 0; k < FB; k++)
			if(k < n) m = fminf(m, fabsf(ld2<COH>(Do + u[k]).x));
		bh = m == INFINITY ? 0.f : m;
		bl = 0.f;
	}
	const float old_rel = vd.x == INFINITY ? INFINITY : 0.f;
	Cand32 best = {old_rel, 0.f, 0.f, 0.f};
	Nb32 first, last;
#pragma unroll
	for(uint32_t c = 0; c < FB; c += FC)
	{
		float2 dk[FC];
		float4 pk[FC];
#pragma unroll
		for(uint32_t q = 0; q < FC; q++)
			if(c + q < n)
			{
				dk[q] = ld2<COH>(Do + u[c + q]);
				pk[q] = __ldg(F.P + u[c + q]);
			}
#pragma unroll
		for(uint32_t q = 0; q < FC; q++)
			if(c + q < n)
			{
				const Nb32 cur = make_nb(pk[q], rel_to(unflag(dk[q]), bh, bl), pv, u[c + q]);
				if(c + q == 0) first = cur;
				else take32<CL, COH>(last, cur, best, lab, Co);
				last = cur;
			}
	}
	if(closed) take32<CL, COH>(last, first, best, lab, Co);
	if(!(best.p < old_rel)) return vd;
	return df_result(bh, bl, best);
}

// ---------------------------------------------------------------------------
// Lean FP32 relaxation (distances only, no labels).
//
// The reference takes, per star triangle, either the planar solution or the
// edge fallback min(t0 + |X0|, t1 + |X1|), then the minimum over the star.
// Where the planar test passes, the planar value is the distance from a
// virtual source S with |S - x0| = t0 and |S - x1| = t1, so by the triangle
// inequality it is <= t0 + |X0| and <= t1 + |X1|.  Hence the minimum over the
// star equals the minimum of (a) every neighbour's edge value t_k + |X_k| and
// (b) the planar values of the triangles whose test passes -- provided every
// neighbour lies on a triangle (two or more fan entries) and no triangle is
// degenerate (the reference ignores a degenerate triangle with finite inputs,
// edge values included).  Each edge value is then formed once per neighbour
// instead of twice per triangle, and a triangle carries no fallback selection.
// A vertex whose star has a degenerate triangle (A^2 not > 0) is relaxed again
// by the triangle-by-triangle path (relax32), so the reference's rule holds
// exactly there.  The two formulations agree to rounding: the only difference
// is which of two candidates equal to within an ulp of an edge is kept.
//
// The padded rows (FAN8_*) make every slot a real neighbour and every star
// triangle a pair of consecutive slots (the closing one too), so the lanes of
// a warp walk the same number of slots -- the warp's longest row -- with no
// per-slot branch: a slot past a lane's own row repeats its last entry, whose
// edge value is already a candidate and whose pair of equal ids is no
// triangle (its planar test compares NaN; it is exempt from the degenerate
// check).
//
// INF neighbours need no test: their relative offset comes out NaN, every
// comparison with it is false, and a NaN offset never passes the planar test
// (max(r, 0) is then 0 and the tests compare NaN), which is the reference's
// "INF inputs take the edge fallback" -- the other neighbour's edge value is
// a candidate of its own.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 rel_to_lean(float2 dv, float bh, float bl)
{
	float h, eh;
	two_sum(dv.x, -bh, h, eh);
	const float l = (dv.y - bl) + eh;
	const float t = h + l;
	return make_float2(t, l - (t - h));
}

// The running best (value, and the operands its exact value is formed from).
struct Best32 {
	float p, t, x, te;
};

__device__ __forceinline__ void take_edge(const Nb32 &k, Best32 &b)
{
	const float d = k.t + k.l;
	if(d < b.p) b = {d, k.t, k.l, k.te};
}

// Planar candidate of triangle (a, b).  A degenerate triangle (A^2 not > 0)
// of two distinct vertices sets best.p to -INF, which no later candidate
// beats and which sends the vertex to the triangle-by-triangle path.
__device__ __forceinline__ void take_planar(const Nb32 &a, const Nb32 &b, bool distinct, Best32 &best)
{
	const float ex = b.x - a.x, ey = b.y - a.y, ez = b.z - a.z;
	const float e2 = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
	const float a1 = -fmaf(a.x, ex, fmaf(a.y, ey, a.z * ez));  // -X0.E
	const float a0 = e2 - a1;                                 // X1.E = E.E + X0.E
	const float q01 = a.q - a1;                               // X0.X1 = X0.X0 + X0.E
	const float cx = fmaf(a.y, b.z, -a.z * b.y);
	const float cy = fmaf(a.z, b.x, -a.x * b.z);
	const float cz = fmaf(a.x, b.y, -a.y * b.x);
	const float A2 = fmaf(cx, cx, fmaf(cy, cy, cz * cz));
	const float dt = (b.t - a.t) + (b.te - a.te);
	const float r = fmaf(-dt, dt, e2);
	const float delta = fmaf(a1, dt, sqrt_a(A2 * fmaxf(r, 0.f))) * rcp_a(e2);
	const float p = a.t + delta;
	if(fmaf(a0, delta, q01 * dt) > 0.f && fmaf(a1, delta, -a.q * dt) > 0.f && !(r < 0.f) && p < best.p)
		best = {p, a.t, delta, a.te};
	if(!(A2 > 0.f) && distinct) best.p = -INFINITY;
}

// The triangle-by-triangle relaxation (reference order and degenerate rule),
// for the rare star with a degenerate triangle.
template <bool COH>
__device__ __noinline__ float2 relax32_exact(const FieldDev &F, uint32_t v, const float2 *Do)
{
	uint32_t lab;
	float2 vd;
	bool skip;
	return relax32<false, COH>(F, v, Do, nullptr, lab, 0u, false, vd, skip);
}

template <bool COH>
__device__ __forceinline__ float2 relax32_lean(const FieldDev &F, uint32_t v, const float2 *Do, uint32_t win_s,
                                               bool try_skip, float2 &vd, bool &skip)
{
	const unsigned am = __activemask();
	const uint4 ra = __ldg(F.fan8 + 2 * (size_t) v), rb = __ldg(F.fan8 + 2 * (size_t) v + 1);
	const float2 vs = ld2<COH>(Do + v);
	vd = unflag(vs);
	const float4 pv = __ldg(F.P + v);
	const uint32_t u[FB] = {ra.x & FAN8_ID_MASK, ra.y, ra.z, ra.w, rb.x, rb.y, rb.z, rb.w};
	const bool ovf = rb.w == FAN8_OVERFLOW;
	const uint32_t n = (ra.x >> FAN8_N_SHIFT) & 15u;
	// slots this lane walks: its row, plus the repeated first neighbour of a closed fan
	const uint32_t m = ovf || n < 2 ? 0u : n + (ra.x >> 31);
	const uint32_t mw = __reduce_max_sync(am, m);  // the warp walks mw slots
	const unsigned live = __ballot_sync(am, m != 0);  // the lanes that go on below
	if(ovf)
	{
		uint32_t lab;
		return relax32_csr<false, COH>(F, v, Do, nullptr, lab, vd, pv);
	}
	if(!m) return vd;  // no triangle
	if(try_skip && __all_sync(live, !flagged(vs.x)))
	{
		bool same = true;
#pragma unroll
		for(uint32_t k = 0; k < FB; k++)
			if(k < mw) same &= u[k] >= win_s && !flagged(ld_d<float, COH>(reinterpret_cast<const float *>(Do + u[k])));
		if(same)
		{
			skip = true;
			return vd;
		}
	}
	float bh = vd.x, bl = vd.y;
	if(bh == INFINITY)
	{
		float mn = INFINITY;
#pragma unroll
		for(uint32_t k = 0; k < FB; k++)
			if(k < mw) mn = fminf(mn, fabsf(ld2<COH>(Do + u[k]).x));
		bh = mn == INFINITY ? 0.f : mn;
		bl = 0.f;
	}
	const float old_rel = vd.x == INFINITY ? INFINITY : 0.f;
	Best32 best = {old_rel, 0.f, 0.f, 0.f};
	Nb32 last;
	// slots in chunks of FC loaded together; the bound mw is the same on every
	// lane, so the tests below are uniform branches
#pragma unroll
	for(uint32_t c = 0; c < FB; c += FC)
	{
		if(c >= mw) break;
		float2 dk[FC];
		float4 pk[FC];
#pragma unroll
		for(uint32_t q = 0; q < FC; q++)
			if(q == 0 || c + q < mw)
			{
				dk[q] = ld2<COH>(Do + u[c + q]);
				pk[q] = __ldg(F.P + u[c + q]);
			}
#pragma unroll
		for(uint32_t q = 0; q < FC; q++)
			if(q == 0 || c + q < mw)
			{
				const Nb32 cur = make_nb_lean(pk[q], rel_to_lean(unflag(dk[q]), bh, bl), pv);
				take_edge(cur, best);
				if(c + q > 0) take_planar(last, cur, u[c + q - 1] != u[c + q], best);
				last = cur;
			}
	}
	if(best.p == -INFINITY) return relax32_exact<COH>(F, v, Do);
	if(!(best.p < old_rel)) return vd;
	return df_result(bh, bl, {best.p, best.t, best.x, best.te});
}

// Relax window vertex v of field F (buffers d -> d^1) and, if v is in the
// check ring (v < chk_e), apply relative_error + is_ok
// (src/cuda/geodesics_ptp.cu:284-299, 371-375).  Returns 1 if v fails
// the test.  COH: distances may have been written by other CTAs of this launch.
template <typename T, bool CL, bool COH>
__device__ __forceinline__ int sweep_vertex(const FieldDev &F, uint32_t d, uint32_t v, uint32_t win_s, uint32_t chk_e,
                                            bool try_skip = false, bool *skipped = nullptr)
{
	const uint32_t *Co = CL ? F.C[d] : nullptr;
	uint32_t lab = 0;
	if constexpr(sizeof(T) == 4)
	{
		const float2 *Do = static_cast<const float2 *>(F.D[d]);
		float2 ov;
		bool skip = false;
		float2 nv;
		if constexpr(!CL && GP_LEAN) nv = relax32_lean<COH>(F, v, Do, win_s, try_skip, ov, skip);
		else nv = relax32<CL, COH>(F, v, Do, Co, lab, win_s, try_skip, ov, skip);
		if(skipped) *skipped = skip;
		const bool chg = __float_as_uint(nv.x) != __float_as_uint(ov.x) || __float_as_uint(nv.y) != __float_as_uint(ov.y);
		static_cast<float2 *>(F.D[d ^ 1u])[v] = make_float2(__uint_as_float(__float_as_uint(nv.x) | (chg ? 0x80000000u : 0u)), nv.y);
		if(v >= chk_e) goto labels;
		if(CL) F.C[d ^ 1u][v] = lab;
		// relative_error + is_ok without the division and in FP32: the change
		// is formed from the hi and lo differences; 0 and INF old values fail
		// as |new - old| / old does (NaN or INF is not < tol).
		const float df = (nv.x - ov.x) + (nv.y - ov.y);
		return !(fabsf(df) < F.tol32 * ov.x);
	}
	else
	{
		const double *Do = static_cast<const double *>(F.D[d]);
		const double nv = relax64<CL, COH>(F, v, Do, Co, lab);
		static_cast<double *>(F.D[d ^ 1u])[v] = nv;
		if(v >= chk_e) goto labels;
		const double o = ld_d<double, COH>(Do + v);
		if(CL) F.C[d ^ 1u][v] = lab;
		// relative_error + is_ok (src/cuda/geodesics_ptp.cu:284-299, 371-375), in FP64
		return !(fabs(nv - o) / o < F.tol);
	}
labels:
	if(CL) F.C[d ^ 1u][v] = lab;
	return 0;
}

// ---------------------------------------------------------------------------
// classify: reset every field's schedule state (i = 1, j = 2, d = 0).  Every
// field starts on one CTA, unless the cost model predicted it outgrows one.
// ---------------------------------------------------------------------------
__global__ void classify_kernel(FieldDev *fields, FieldState *state, uint32_t n_fields, uint32_t local_window,
                                const uint32_t *pred_big)
{
	const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
	if(warp >= n_fields) return;
	const FieldDev &F = fields[warp];
	FieldState &st = state[warp];
	const uint32_t nl = st.n_limits;
	if(lane == 0)
	{
		st.big = 0;
		st.nr = nl ? F.limits[nl - 1] : 0;
		st.i = 1;
		st.j = 2;
		st.d = 0;
		st.iter = 0;
		st.n_iter = 0;
		st.live = 0;
		st.relax = 0;
		st.max_iter = F.max_iter ? F.max_iter : (nl << 1);
		st.n_limits = nl;
		if(F.stream)
		{
			// toplesets still to come: the grid launch builds them, then opens
			// the first window (n_limits, nr and max_iter are set there)
			st.nr = 0;
			st.big = 1;
			st.live = 1;
			return;
		}
		// a field the cost model expects to outgrow one CTA starts on the grid
		// launch right away (its first sweep opened here)
		if(pred_big && pred_big[warp] && nl >= 3)
		{
			open_sweep(F, st, true);
			st.big = st.live;
		}
	}
	(void) local_window;
}

// ---------------------------------------------------------------------------
// Cost-model features of every field (one warp per field), from its toplesets
// and its mesh's geometry statistics; the 16 values of GP_MLP_IN.
// ---------------------------------------------------------------------------
__global__ void field_features_kernel(const FieldDev *fields, const FieldState *state, uint32_t n_fields, float *out)
{
	const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
	if(warp >= n_fields) return;
	const FieldDev &F = fields[warp];
	const uint32_t nl = state[warp].n_limits;
	const uint32_t L = nl ? nl - 1 : 0;
	const uint32_t *lim = F.limits;
	uint32_t rmax = 0, amax = 0, bound = 0;
	for(uint32_t k = lane; k < L; k += 32)
	{
		const uint32_t r = lim[k + 1] - lim[k];
		if(r > rmax) { rmax = r; amax = k; }
	}
	for(uint32_t j = 2 + lane; j < nl; j += 32) bound = max(bound, lim[j] - lim[j >> 1]);
	for(int o = 16; o; o >>= 1)
	{
		const uint32_t r2 = __shfl_xor_sync(0xffffffffu, rmax, o), a2 = __shfl_xor_sync(0xffffffffu, amax, o);
		if(r2 > rmax || (r2 == rmax && a2 < amax)) { rmax = r2; amax = a2; }
		bound = max(bound, __shfl_xor_sync(0xffffffffu, bound, o));
	}
	if(lane) return;
	const uint32_t nr = nl ? lim[nl - 1] : 0;
	auto ring = [&](uint32_t k) { return k < L ? (float) (lim[k + 1] - lim[k]) : 0.f; };
	const float Lf = (float) max(L, 1u);
	float *x = out + (size_t) warp * MLP_IN;
	x[0] = logf((float) max(F.m.nv, 1u));
	x[1] = logf(Lf);
	x[2] = logf((float) max(F.ns, 1u));
	x[3] = logf((float) max(rmax, 1u));
	x[4] = logf(fmaxf((float) nr / Lf, 1.f));
	x[5] = (float) amax / Lf;
	x[6] = logf((float) bound + 1.f);
	x[7] = logf(ring(L / 4) + 1.f);
	x[8] = logf(ring(L / 2) + 1.f);
	x[9] = logf(ring(3 * L / 4) + 1.f);
	x[10] = F.m.stats[0];
	x[11] = F.m.stats[1];
	x[12] = F.m.stats[2];
	x[13] = F.m.stats[3];
	x[14] = F.m.stats[4];
	x[15] = (float) nr / (float) max(F.m.nv, 1u);
}

// Predictions -> start mode and local queue order (one CTA).  Predicted
// sweeps s = rings * exp(y0), relaxations r = vertices * exp(y1); a field
// whose mean window r / s exceeds local_window starts on the grid launch; the
// others are queued longest predicted chain first (s * ceil(window / LT)).
__global__ void __launch_bounds__(1024) plan_kernel(const FieldDev *fields, const FieldState *state, uint32_t n_fields,
                                                    const float *pred, uint32_t local_window, uint32_t lt,
                                                    uint32_t *pred_big, float *cost, uint32_t *perm)
{
	for(uint32_t f = threadIdx.x; f < n_fields; f += blockDim.x)
	{
		const uint32_t nl = state[f].n_limits;
		const float L = (float) (nl ? nl - 1 : 1);
		const float sw = fmaxf(L * expf(pred[2 * f]), 1.f);
		const float rx = (float) fields[f].m.nv * expf(pred[2 * f + 1]);
		const float win = rx / sw;
		const uint32_t big = nl >= 3 && win > (float) local_window;
		const float c = sw * fmaxf(1.f, ceilf(win / (float) lt));
		pred_big[f] = big;
		cost[f] = big ? -1.f : (c == c ? c : 0.f);  // a NaN cost would break the ranking
	}
	__syncthreads();
	for(uint32_t f = threadIdx.x; f < n_fields; f += blockDim.x)
	{
		const float c = cost[f];
		uint32_t rank = 0;
		for(uint32_t g = 0; g < n_fields; g++)
		{
			const float d = cost[g];
			rank += d > c || (d == c && g < f);
		}
		perm[rank] = f;
	}
}


// ---------------------------------------------------------------------------
// One CTA sweeps one field (run_ptp_gpu's loop, src/cuda/geodesics_ptp.cu:
// 198-229): the window is swept in CTA-sized chunks and __syncthreads_or()
// both merges the ring-i test and separates the sweeps.  Every thread keeps
// the schedule in registers.  When the next window would exceed
// local_window vertices the field is handed, mid-schedule, to the grid-wide
// launch (state saved with that sweep already opened, big = 1).
// ---------------------------------------------------------------------------
constexpr int LT = 512;

template <typename T, bool CL>
__global__ void __launch_bounds__(LT) ptp_local_kernel(FieldDev *fields, FieldState *state, uint32_t n_fields,
                                                       uint32_t *queue, uint32_t local_window, const uint32_t *perm)
{
	__shared__ uint32_t s_f;
	for(;;)
	{
		if(threadIdx.x == 0)
		{
			const uint32_t q = atomicAdd(queue, 1u);
			s_f = q < n_fields && perm ? perm[q] : q;
		}
		__syncthreads();
		const uint32_t f = s_f;
		__syncthreads();
		if(f >= n_fields) return;
		FieldState &gst = state[f];
		if(gst.n_limits < 3 || gst.big) continue;
		const FieldDev &F = fields[f];
		FieldState st = {};
		st.i = 1;
		st.j = 2;
		st.max_iter = gst.max_iter;
		st.n_limits = gst.n_limits;
		open_sweep(F, st, threadIdx.x == 0);
		while(st.live && st.win_e - st.win_s <= local_window)
		{
			int bad = 0;
			for(uint32_t v = st.win_s + threadIdx.x; v < st.win_e; v += LT)
				bad |= sweep_vertex<T, CL, false>(F, st.d, v, st.win_s, st.chk_e);
			close_sweep(st, !__syncthreads_or(bad));
			open_sweep(F, st, threadIdx.x == 0);
		}
		if(threadIdx.x == 0)
		{
			gst.i = st.i;
			gst.j = st.j;
			gst.d = st.d;
			gst.iter = st.iter;
			gst.n_iter = st.n_iter;
			gst.relax = st.relax;
			gst.live = st.live;
			gst.win_s = st.win_s;
			gst.win_e = st.win_e;
			gst.chk_e = st.chk_e;
			gst.big = st.live;  // still running: the grid-wide launch continues it
		}
	}
}

// ---------------------------------------------------------------------------
// Grid-wide persistent sweeps of the fields handed over by ptp_local_kernel,
// all in lockstep.  Every CTA holds the schedule of every field in shared
// memory and applies the reference's rule itself after each barrier (the
// rule is deterministic, so all copies agree); the only cross-CTA data per
// step are the ring-i flags, triple-buffered so that they can be cleared
// without an extra barrier.  A step: walk the tiles of all live windows ->
// counting barrier -> read the flags, advance, re-plan.
// ---------------------------------------------------------------------------
struct GridArgs {
	FieldDev *fields;
	FieldState *state;
	uint32_t n_fields;
	uint32_t *notok;  // 3 * n_fields, zeroed before the launch
	uint32_t *bar;    // GRID_BAR_WORDS, zeroed: see count_barrier
	unsigned long long *steps;  // null, or 2 words per step: start time (ns), tiles << 32 | live fields
	uint32_t steps_cap;
	const QCtl *ctl;            // null, or the launch-mode choice (runs only if mode == GRID_LOCKSTEP)
	uint32_t spin_limit;        // polls before a barrier wait gives up
	uint32_t phantom;           // arrivals the barrier waits for beyond the launch's CTAs (0; tests)
	// streamed fields (see stream_worker): their ids, the worker CTAs at the end
	// of the launch, per-field progress words and the snapshot CTA 0 takes of them
	const uint32_t *sids;
	uint32_t n_stream;
	uint32_t workers;
	uint32_t ctas;              // sweeping CTAs: the launch's CTAs minus the workers
	unsigned long long *sprog;  // n_stream, zeroed
	unsigned long long *snap;   // ptp_snap_words(n_fields): see SNAP_DONE
	// a launch that resumes after a streaming launch: that launch's barrier
	// words (nothing to do if it gave up; its step count offsets the trace)
	const uint32_t *prev;
};

__device__ __forceinline__ unsigned long long global_ns()
{
	unsigned long long t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}

struct SchedSmem {
	// live: bit 0 = a window is open this step; for a streamed field also bits
	// 24-31 = its index in GridArgs::sids + 1, bits 8-9 = wait (1: the first
	// window is not open yet, 2: a sweep is done and the next window waits for
	// the rings it reads), bit 16 = that sweep's ring test passed.  (Packed: the
	// entry stays 64 bytes, whose loads in the sweep loop are aligned.)
	uint32_t i, j, d, iter, n_iter, max_iter, nl, live, win_s, win_e, chk_e;
	// limits the next window may need, loaded while this step runs:
	// [0..1] from i' = max(i, j'/2) (ring test failed), [2..3] from
	// max(i + 1, j'/2) (passed), [4] at j' (the next j)
	uint32_t nx[5];
};

__device__ __forceinline__ uint32_t sched_sq(const SchedSmem &x) { return x.live >> 24; }  // 0: not streamed
__device__ __forceinline__ uint32_t sched_wait(const SchedSmem &x) { return (x.live >> 8) & 3u; }

// The limits the next boundary may need, loaded while the step runs (plain
// loads).  Not for a streamed field: its limits are written during the launch,
// and a line of them in this SM's L1 could be stale; its windows open through
// open_sweep, which loads from L2.  Once its toplesets are done it becomes a
// plain field (stream_boundary), and from then on its lines, which no plain
// load touched before (field bases are 128-byte aligned in such a launch),
// come fresh from L2.  (An L2-load branch here instead raised the sweep
// loop's spills: grid phase +10 %.)
template <bool STREAM>
__device__ __forceinline__ void prefetch_limits(const FieldDev &F, SchedSmem &x)
{
	if(!(x.live & 1u) || (STREAM && sched_sq(x))) return;
	const uint32_t j1 = x.j < x.nl - 1 ? x.j + 1 : x.j;
	const uint32_t ia = max(x.i, j1 >> 1), ib = max(x.i + 1, j1 >> 1);
	const uint32_t *lim = F.limits;
	x.nx[0] = ia < x.nl ? lim[ia] : 0u;
	x.nx[1] = ia + 1 < x.nl ? lim[ia + 1] : 0u;
	x.nx[2] = ib < x.nl ? lim[ib] : 0u;
	x.nx[3] = ib + 1 < x.nl ? lim[ib + 1] : 0u;
	x.nx[4] = lim[j1];
}

// open_sweep with the prefetched limits; `passed` = the ring test of the
// sweep just closed passed (close_sweep advanced i)
__device__ __forceinline__ void open_sweep_cached(const FieldDev *F, FieldState &st, const SchedSmem &x, bool passed)
{
	if(st.i < st.j && st.iter < st.max_iter)
	{
		st.iter++;
		if(st.i < (st.j >> 1)) st.i = st.j >> 1;
		st.win_s = passed ? x.nx[2] : x.nx[0];
		st.chk_e = passed ? x.nx[3] : x.nx[1];
		st.win_e = x.nx[4];
		st.live = 1;
		if(F && F->trace && st.n_iter < F->trace_cap)
		{
			F->trace[2 * st.n_iter] = st.i;
			F->trace[2 * st.n_iter + 1] = st.j;
		}
	}
	else st.live = 0;
}

// Counting barrier: every CTA arrives with a fire-and-forget release add on
// one counter and waits with an acquire spin until all CTAs of the step have
// arrived.  (A two-level form, CTAs counted on 16 group counters whose last
// arrival then signals the top counter, needs a returning atomic per CTA:
// one more L2 round trip per step, measured 2-13 % slower.)  Bounded: gives
// up after `limit` polls (error bit set, abort raised, caller returns).
// bar: [0] arrivals, [1] abort, [2] error bits, [3] steps, [4..5] skip count.

__device__ __forceinline__ bool count_barrier(uint32_t *bar, uint32_t step, uint32_t limit, uint32_t phantom,
                                              uint32_t ctas)
{
	__shared__ uint32_t s_ok;
	__syncthreads();
	if(threadIdx.x == 0)
	{
		s_ok = 1;
		asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(bar) : "memory");
		const uint32_t target = (ctas + phantom) * (step + 1);
		uint32_t spins = 0;
		while(ld_acquire(bar) < target)
		{
			// another CTA's abort is looked for every 32 polls (one load per poll)
			if(++spins > limit || ((spins & 31u) == 0 && ld_relaxed(bar + 1)))
			{
				atomicOr(bar + 2, DEV_ERR_TIMEOUT);
				atomicExch(bar + 1, 1u);
				s_ok = 0;
				break;
			}
		}
	}
	__syncthreads();
	return s_ok != 0;
}

// Tiles of every live window (TV window vertices per tile); ts[G] = total.
template <uint32_t TV, bool STREAM>
__device__ __forceinline__ void grid_plan(const SchedSmem *fs, uint32_t *ts, uint32_t G, uint32_t *s_tile)
{
	if(G <= NT)
	{
		// one round (the usual case): one block scan, the tile counter reset with it
		const uint32_t q = threadIdx.x;
		const uint32_t tiles = q < G && (STREAM ? (fs[q].live & 1u) : fs[q].live) ? (fs[q].win_e - fs[q].win_s + TV - 1) / TV : 0u;
		uint32_t tot;
		const uint32_t ex = block_exclusive_scan<NT>(tiles, &tot);
		if(q < G) ts[q] = ex;
		if(q == 0)
		{
			ts[G] = tot;
			*s_tile = 0;
		}
		__syncthreads();
		return;
	}
	__shared__ uint32_t carry;
	if(threadIdx.x == 0)
	{
		carry = 0;
		*s_tile = 0;
	}
	__syncthreads();
	for(uint32_t base = 0; base < G; base += NT)
	{
		const uint32_t q = base + threadIdx.x;
		const uint32_t tiles = q < G && (STREAM ? (fs[q].live & 1u) : fs[q].live) ? (fs[q].win_e - fs[q].win_s + TV - 1) / TV : 0u;
		uint32_t tot;
		const uint32_t ex = block_exclusive_scan<NT>(tiles, &tot);
		if(q < G) ts[q] = carry + ex;
		__syncthreads();
		if(threadIdx.x == 0) carry += tot;
		__syncthreads();
	}
	if(threadIdx.x == 0) ts[G] = carry;
	__syncthreads();
}

// ---------------------------------------------------------------------------
// Streamed fields: toplesets and ring renumbering inside the lockstep launch.
//
// The BFS of a field on a large mesh is a chain of levels (~5 us each on one
// CTA: dependent L2 round trips and CTA barriers) as long as the field has
// rings, and without streaming the field's sweeps start only after it ends.
// But a sweep reads only the rings up to j + 1, and the sweeps advance about
// one ring per grid step (tens of microseconds), far slower than the BFS.  So
// the last `workers` CTAs of the launch build the toplesets of the streamed
// fields -- up to STREAM_PER_WORKER each, one level of each in turn -- and
// renumber every ring as soon as the next ring is known, publishing per field
// the rings and positions done; the other CTAs sweep.  A streamed field opens
// its next window only when the renumbered part covers every position the
// window reads plus STREAM_MARGIN: the sweeps read positions and fan rows
// through L1, which other SMs' writes do not update, so no 128-byte line a
// sweep touches may still change (field bases are aligned to STREAM_ALIGN
// slots for the same reason).  The readiness every sweeping CTA acts on is a
// snapshot CTA 0 takes at the start of the step (before its arrival at the
// step's barrier), so all copies of the schedules take the same decisions; a
// field that waits just skips steps.  The sweeps are the same sweeps in the
// same order as without
// streaming, so the results are bit-identical.  Once every worker is done
// (the first boundary whose snapshot counts them all), the launch writes every
// schedule back to its FieldState and ends; a launch of the plain lockstep
// kernel, which starts from the FieldState, sweeps the rest on every SM and
// with the plain kernel's code.
// ---------------------------------------------------------------------------
constexpr uint32_t STREAM_DONE = 0x80000000u;  // progress: rings renumbered | DONE (high word), positions (low)
constexpr unsigned long long STREAM_WAIT_NS = 2000000000ull;  // 2 s of steps without any window ready
// GridArgs::snap: [0, 2 * STREAM_MAX) the progress snapshots of the two step
// parities, then (zeroed before the launch) the workers done as CTA 0 saw them
// at the start of a step of parity p ([SNAP_DONE + p]) and the workers done
// ([SNAP_WORKERS]).
constexpr uint32_t SNAP_DONE = 2 * STREAM_MAX, SNAP_WORKERS = SNAP_DONE + 2;
constexpr uint32_t SNAP_WORDS = SNAP_DONE + 4, SNAP_CTL_WORDS = 4;

// Ring positions [k0, k1) of streamed field F: the FP32 sweeps' padded fan
// rows, positions and initial distances, as fill_kernel writes them.  The
// first chunk's vertex and mesh rows (position k0 + threadIdx.x) come from
// the caller, which loaded them for the same positions in the level's
// discover pass: one dependent L2 trip fewer per ring.
__device__ __forceinline__ void stream_renumber(const FieldDev &F, uint32_t k0, uint32_t k1, uint32_t v0,
                                                uint4 ra0, uint4 rb0)
{
	float2 *D0 = static_cast<float2 *>(F.D[0]);
	float2 *D1 = static_cast<float2 *>(F.D[1]);
	for(uint32_t k = k0 + threadIdx.x; k < k1; k += NT)
	{
		uint32_t v = v0;
		uint4 ra = ra0, rb = rb0;
		if(k >= k0 + NT)
		{
			v = ldcg(F.sorted + k);
			ra = __ldg(F.m.fan8 + 2 * (size_t) v);
			rb = __ldg(F.m.fan8 + 2 * (size_t) v + 1);
		}
		uint32_t r[8], n = 0;
#pragma unroll
		for(uint32_t q = 0; q < 8; q++)
		{
			const uint32_t u = slot_of(ra, rb, q);
			r[q] = FAN8_EMPTY;
			if(u != FAN8_EMPTY)
			{
				r[q] = ldcg(F.inv + u) - 1;  // every neighbour of a ring is in a ring already emitted
				n = q + 1;
			}
		}
		const bool cl = n && (ra.x & FAN_CLOSED);
		if(n)
		{
			const uint32_t pad = cl ? r[0] : r[n - 1];
#pragma unroll
			for(uint32_t q = 1; q < 8; q++)
				if(q >= n) r[q] = pad;
		}
		r[0] = n ? (r[0] & FAN8_ID_MASK) | (n << FAN8_N_SHIFT) | (cl ? FAN_CLOSED : 0u) : 0u;
		F.fan8[2 * (size_t) k] = make_uint4(r[0], r[1], r[2], r[3]);
		F.fan8[2 * (size_t) k + 1] = make_uint4(r[4], r[5], r[6], r[7]);
		F.P[k] = __ldg(F.m.pos + v);
		const float2 d0 = make_float2(k < F.ns ? 0.f : -INFINITY, 0.f);  // all but the sources flagged
		D0[k] = d0;
		D1[k] = d0;
	}
}

// The sentinel slot nr (every unreached vertex reads it): no fan, distance INF.
__device__ __forceinline__ void stream_sentinel(const FieldDev &F, uint32_t nr)
{
	F.fan8[2 * (size_t) nr] = make_uint4(0u, FAN8_EMPTY, FAN8_EMPTY, FAN8_EMPTY);
	F.fan8[2 * (size_t) nr + 1] = make_uint4(FAN8_EMPTY, FAN8_EMPTY, FAN8_EMPTY, FAN8_EMPTY);
	F.P[nr] = make_float4(0.f, 0.f, 0.f, 0.f);
	static_cast<float2 *>(F.D[0])[nr] = make_float2(INFINITY, 0.f);
	static_cast<float2 *>(F.D[1])[nr] = make_float2(INFINITY, 0.f);
}

// One worker CTA: the toplesets of streamed fields w, w + workers, ... (the
// one-CTA BFS of gp_toplesets.cu, same keys and order), one level of each in
// turn; after level L (ring L + 1 emitted, with its new ids) ring L is
// renumbered and the progress published (release): rings 0..L and positions
// [0, limits[L + 1]).  The last level also writes the sentinel, n_limits and
// nr, then publishes DONE.  Leaves early if the sweeping CTAs gave up.
__device__ __noinline__ void stream_worker(const GridArgs &a, uint32_t w)
{
	// (no frontier copies in shared memory: any shared memory of this function
	// is reserved on every SM of the launch and costs the sweeps L1 capacity)
	__shared__ uint32_t wst[STREAM_PER_WORKER][4];  // level, s, e, live
	__shared__ uint32_t s_abort;
	const uint32_t W = a.workers;
	uint32_t nf = 0;
	for(uint32_t q = w; q < a.n_stream && nf < STREAM_PER_WORKER; q += W) nf++;
	for(uint32_t t = 0; t < nf; t++)
	{
		const uint32_t f = a.sids[w + t * W];
		const FieldDev &F = a.fields[f];
		const bool live = a.state[f].bfs_live != 0;  // 0: a source outside the mesh (seed)
		const uint32_t ns = live ? F.ns : 0u;
		for(uint32_t k = threadIdx.x; k < ns; k += NT)
			atomicMax(F.inv + ldcg(F.sorted + k), k + 1);  // repeated sources: the last occurrence
		if(threadIdx.x == 0)
		{
			wst[t][0] = 0;
			wst[t][1] = 0;
			wst[t][2] = ns;
			wst[t][3] = live;
			if(!live)
			{
				// no toplesets: the gather reads the sentinel at slot 0
				stream_sentinel(F, 0);
				a.state[f].nr = 0;
			}
		}
		__syncthreads();
		if(!live && threadIdx.x == 0) st_release(a.sprog + w + t * W, (unsigned long long) STREAM_DONE << 32);
	}
	__syncthreads();
	for(;;)
	{
		bool any = false;
		for(uint32_t t = 0; t < nf; t++)
		{
			__syncthreads();
			if(!wst[t][3]) continue;  // uniform: read after the barrier
			any = true;
			const uint32_t q = w + t * W, f = a.sids[q];
			const FieldDev &F = a.fields[f];
			const uint32_t level = wst[t][0], s = wst[t][1];
			uint32_t e = wst[t][2];
			// pass 1: discover (the first frontier chunk's rows kept in registers)
			uint4 ra = make_uint4(FAN8_EMPTY, FAN8_EMPTY, FAN8_EMPTY, FAN8_EMPTY), rb = ra;
			uint32_t v0 = 0, c0 = 0;
			if(s + threadIdx.x < e)
			{
				const uint32_t p = s + threadIdx.x;
				v0 = ldcg(F.sorted + p);
				ra = __ldg(F.m.fan8 + 2 * (size_t) v0);
				rb = __ldg(F.m.fan8 + 2 * (size_t) v0 + 1);
				c0 = discover_local(F, p, v0, ra, rb);
			}
			for(uint32_t p = s + NT + threadIdx.x; p < e; p += NT)
			{
				const uint32_t v = ldcg(F.sorted + p);
				discover_local(F, p, v, __ldg(F.m.fan8 + 2 * (size_t) v), __ldg(F.m.fan8 + 2 * (size_t) v + 1));
			}
			__syncthreads();
			// pass 2: count, scan in frontier order, emit with the new ids
			uint32_t carry = 0;
			for(uint32_t base = s, c = 0; base < e; base += NT, c++)
			{
				const uint32_t p = base + threadIdx.x;
				uint32_t v = 0, cnt = 0, mask = 0, cand = 0xFFu;
				uint4 x0 = make_uint4(FAN8_EMPTY, FAN8_EMPTY, FAN8_EMPTY, FAN8_EMPTY), x1 = x0;
				if(p < e)
				{
					if(c == 0)
					{
						v = v0;
						x0 = ra;
						x1 = rb;
						cand = c0;
					}
					else
					{
						v = ldcg(F.sorted + p);
						x0 = __ldg(F.m.fan8 + 2 * (size_t) v);
						x1 = __ldg(F.m.fan8 + 2 * (size_t) v + 1);
					}
					mask = owned(F, p, v, x0, x1, cnt, cand);
				}
				uint32_t tot;
				const uint32_t ex = block_exclusive_scan<NT>(cnt, &tot);
				uint32_t o = carry + ex;
#pragma unroll
				for(uint32_t k = 0; k < 8; k++)
					if(mask & (1u << k))
					{
						const uint32_t u = slot_of(x0, x1, k);
						F.sorted[e + o] = u;
						F.ring[u] = level + 1;
						F.inv[u] = e + o + 1;
						o++;
					}
				carry += tot;
			}
			__syncthreads();
			// ring `level` = [s, e): all its neighbours have their new ids now
			stream_renumber(F, s, e, v0, ra, rb);
			__syncthreads();
			if(threadIdx.x == 0)
			{
				if(carry && e + carry > F.cap_sorted)
				{
					// more vertices than the field holds: a broken mesh table; end the
					// field here (its sweeps see n_limits = 0) and report it
					carry = 0;
					e = 0;
					a.state[f].status |= DEV_ERR_BOUNDS;
					atomicOr(a.bar + 2, DEV_ERR_BOUNDS);
				}
				if(carry)
				{
					F.limits[level + 2] = e + carry;
					wst[t][0] = level + 1;
					wst[t][1] = e;
					wst[t][2] = e + carry;
					st_release(a.sprog + q, ((unsigned long long) (level + 1) << 32) | e);
				}
				else
				{
					stream_sentinel(F, e);
					a.state[f].n_limits = e ? level + 2 : 0u;
					a.state[f].nr = e;
					a.state[f].bfs_live = 0;
					wst[t][3] = 0;
					st_release(a.sprog + q, ((unsigned long long) (STREAM_DONE | (level + 1)) << 32) | (e + 1));
				}
			}
		}
		if(threadIdx.x == 0) s_abort = ld_relaxed(a.bar + 1);  // the sweeping CTAs gave up
		__syncthreads();
		if(!any || s_abort) break;
	}
}

// A streamed field at a step boundary (every sweeping CTA, same snapshot):
// takes the ring test of a sweep just done, then returns -2 if the next
// window still waits for its rings, -1 if the field is retired (or has no
// sweep at all), 1 to open its first window, 0 to close and open as usual.
__device__ __forceinline__ int stream_boundary(const GridArgs &a, SchedSmem &x, uint32_t f, const uint32_t *flags,
                                            uint32_t step, bool *passed)
{
	if(!(x.live & 1u) && !sched_wait(x)) return -1;  // retired
	if(x.live & 1u)
		x.live = (x.live & 0xFF000000u) | (2u << 8) | (ldcg(flags + f) ? 0u : 1u << 16);
	// ready: rings up to j + 1 renumbered, and the positions every window
	// after this boundary reads (below limits[j + 2]) plus the margin
	const unsigned long long pr = ldcg(a.snap + (step & 1) * STREAM_MAX + sched_sq(x) - 1);
	const uint32_t rn = (uint32_t) (pr >> 32) & ~STREAM_DONE;
	const bool done = ((pr >> 32) & STREAM_DONE) != 0;
	const FieldDev &Fd = a.fields[f];
	bool ready = done;
	if(!done && rn >= x.j + 2) ready = (uint32_t) pr >= ldcg(Fd.limits + x.j + 2) + STREAM_MARGIN;
	if(!ready) return -2;
	x.nl = done ? ldcg(&a.state[f].n_limits) : rn + 1;
	x.max_iter = Fd.max_iter ? Fd.max_iter : x.nl << 1;
	const uint32_t w = sched_wait(x);
	*passed = (x.live >> 16) & 1u;
	// neither open nor waiting (open_sweep sets bit 0 again); a field whose
	// toplesets are done is a plain field from here on (every CTA decides this
	// on the same snapshot)
	x.live &= done ? 0u : 0xFF000000u;
	if(x.nl < 3) return -1;  // no sweep (the reference's loop needs three limits)
	return w == 1 ? 1 : 0;
}

template <typename T, bool CL, bool STREAM>
__global__ void __launch_bounds__(NT, GP_GRID_MINB) ptp_kernel(GridArgs a)
{
	extern __shared__ __align__(16) unsigned char smem[];
	const uint32_t F = a.n_fields;
	// compacted: entry q describes field id[q]; only fields handed to the grid.
	// Layout: 8-byte counters first, then 4-byte-aligned arrays.
	if(a.ctl && a.ctl->mode != GRID_LOCKSTEP) return;
	if(!STREAM && a.prev && ld_relaxed(a.prev + 1)) return;  // resuming after a launch that gave up
	if constexpr(STREAM)
		if(blockIdx.x >= a.ctas)
		{
			stream_worker(a, blockIdx.x - a.ctas);
			if(threadIdx.x == 0)
			{
				__threadfence();
				atomicAdd(a.snap + SNAP_WORKERS, 1ull);  // this worker's fields are all done
			}
			return;
		}
	// the sweeping CTAs: the whole launch, or (streaming) all but the workers
	const uint32_t C = STREAM ? a.ctas : gridDim.x;
	unsigned long long *rx = reinterpret_cast<unsigned long long *>(smem);
	SchedSmem *fs = reinterpret_cast<SchedSmem *>(rx + F);
	uint32_t *ts = reinterpret_cast<uint32_t *>(fs + F);
	uint32_t *id = ts + F + 1;
	__shared__ uint32_t s_G;
	__shared__ uint32_t s_sj;  // (streaming) the launch ends after this step; ~0u: not yet
	const uint32_t lane = threadIdx.x & 31;
	constexpr uint32_t TV = 32;  // window vertices per tile: one warp's worth

	if(threadIdx.x == 0)
	{
		s_G = 0;
		if(STREAM) s_sj = ~0u;
	}
	__syncthreads();
	bool waiting = false;  // (streaming) a streamed field waits for its rings
	for(uint32_t base = 0; base < F; base += NT)
	{
		const uint32_t f = base + threadIdx.x;
		const bool on = f < F && a.state[f].big && a.state[f].live;
		uint32_t tot;
		const uint32_t ex = block_exclusive_scan<NT>(on ? 1u : 0u, &tot);
		if(on)
		{
			const FieldState &g = a.state[f];
			const uint32_t q = s_G + ex;
			SchedSmem &x = fs[q];
			id[q] = f;
			x.live = 1;
			x.i = g.i;
			x.j = g.j;
			x.d = g.d;
			x.iter = g.iter;
			x.n_iter = g.n_iter;
			x.max_iter = g.max_iter;
			x.nl = g.n_limits;
			x.win_s = g.win_s;
			x.win_e = g.win_e;
			x.chk_e = g.chk_e;
			if constexpr(STREAM)
				if(a.fields[f].stream)
				{
					x.live = (a.fields[f].stream << 24) | (1u << 8);  // waits to open its first window
					waiting = true;
				}
			rx[q] = g.relax;
		}
		__syncthreads();
		if(threadIdx.x == 0) s_G += tot;
		__syncthreads();
	}
	// (streaming) some streamed field waits for rings: set at the boundary of
	// step s in [(s + 1) & 1], read at the top of step s + 1 (kept in shared
	// memory, out of the sweep loop's registers)
	__shared__ uint32_t s_wait[2];
	__shared__ unsigned long long s_idle;            // (streaming) thread 0: start of a run of steps without tiles
	if constexpr(STREAM)
	{
		waiting = __syncthreads_or(waiting);
		if(threadIdx.x == 0)
		{
			s_wait[0] = waiting;
			s_wait[1] = 0;
			s_idle = 0;
		}
	}
	const uint32_t G = s_G;
	__shared__ uint32_t s_tile;  // the CTA's next tile (see the step loop)
	uint32_t n_skip = 0;  // this thread's relaxations skipped as unchanged (summed into bar[4..5] at the end)
	grid_plan<TV, STREAM>(fs, ts, G, &s_tile);
	for(uint32_t q = threadIdx.x; q < G; q += NT) prefetch_limits<STREAM>(a.fields[id[q]], fs[q]);

	for(uint32_t step = 0;; step++)
	{
		const uint32_t total = ts[G];
		if(blockIdx.x == 0 && threadIdx.x == 0 && a.steps)
		{
			// a launch resuming after a streaming launch continues its trace
			const uint32_t k = step + (a.prev ? a.prev[3] : 0u);
			if(k < a.steps_cap)
			{
				uint32_t live = 0;
				for(uint32_t q = 0; q < G; q++) live += fs[q].live & 1u;
				a.steps[2 * k] = global_ns();
				a.steps[2 * k + 1] = ((unsigned long long) total << 32) | live;
			}
		}
		if(!total && (!STREAM || !s_wait[step & 1]))
		{
			if(blockIdx.x == 0 && threadIdx.x == 0) a.bar[3] = step;
			const uint32_t w = __reduce_add_sync(0xffffffffu, n_skip);
			if(lane == 0 && w) atomicAdd(reinterpret_cast<unsigned long long *>(a.bar + 4), (unsigned long long) w);
			break;
		}
		if constexpr(STREAM)
			if(threadIdx.x == 0)
			{
				// s_wait[(step - 1) & 1] was read at the top of the previous step
				s_wait[(step + 1) & 1] = 0;
				// every worker done at the previous step's snapshot: the launch ends
				// after this step's boundary (read there, after the barrier)
				if(s_sj == ~0u && a.workers && ldcg(a.snap + SNAP_DONE + ((step - 1) & 1)) == a.workers) s_sj = step;
				// steps without tiles only while streamed fields wait for rings: bounded
				if(total) s_idle = 0;
				else if(!s_idle) s_idle = global_ns();
				else if(global_ns() - s_idle > STREAM_WAIT_NS)
				{
					atomicOr(a.bar + 2, DEV_ERR_TIMEOUT);
					atomicExch(a.bar + 1, 1u);
				}
			}
		// (streaming) the workers' progress every CTA acts on at this step's
		// boundary: taken before CTA 0's tiles, so that its loads do not delay
		// CTA 0's arrival at the barrier
		if constexpr(STREAM)
			if(blockIdx.x == 0 && threadIdx.x < a.n_stream)
			{
				a.snap[(step & 1) * STREAM_MAX + threadIdx.x] = ld_acquire(a.sprog + threadIdx.x);
				if(threadIdx.x == 0) a.snap[SNAP_DONE + (step & 1)] = ld_acquire(a.snap + SNAP_WORKERS);
			}
		uint32_t *flags = a.notok + (step % 3) * F;
		const bool heavy = total >= C * (NT / 32);  // see unflag: skip only in throughput-bound steps
		uint32_t lo = 0;  // entry of the warp's current tile; tiles only move forward
		// CTA b (one per SM) owns tiles b, b + C, b + 2C, ...; its 32 warps take
		// them in order from a shared counter (reset by grid_plan), so they all
		// finish within about one tile of each other (dealt statically, warps of
		// one SM finished ~10 us apart in a heavy step: the scheduler favours
		// some warps)
		for(;;)
		{
			uint32_t r = 0;
			if(lane == 0) r = atomicAdd(&s_tile, 1u);
			r = __shfl_sync(0xffffffffu, r, 0);
			const uint32_t k = blockIdx.x + r * C;
			if(k >= total) break;
			// last entry whose first tile <= k: the lanes test 32 entries at once
			for(;;)
			{
				const uint32_t q = lo + lane;
				const unsigned m = __ballot_sync(0xffffffffu, q < G && ts[q] <= k);
				const uint32_t c = __popc(m);  // a prefix of the lanes
				lo += c - 1;
				if(c < 32) break;
			}
			const SchedSmem &x = fs[lo];
			const uint32_t f = id[lo];
			int bad = 0;
			bool sk = false;
			const uint32_t v = x.win_s + (k - ts[lo]) * TV + lane;
			if(v < x.win_e) bad = sweep_vertex<T, CL, true>(a.fields[f], x.d, v, x.win_s, x.chk_e, heavy, &sk);
			n_skip += sk;
			// one atomic per warp that saw a failure, no block barrier per tile
			if(__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(flags + f, 1u);
		}
		if(!count_barrier(a.bar, step, a.spin_limit, a.phantom, C)) return;
		// every CTA advances its own copy of every schedule
		for(uint32_t q = threadIdx.x; q < G; q += NT)
		{
			SchedSmem &x = fs[q];
			const uint32_t f = id[q];
			if(blockIdx.x == 0) a.notok[((step + 2) % 3) * F + f] = 0;
			bool passed, open_first = false;
			const bool streamed = STREAM && sched_sq(x);
			if(streamed)
			{
				const int r = stream_boundary(a, x, f, flags, step, &passed);
				if(r < 0)
				{
					if(r == -2) s_wait[(step + 1) & 1] = 1;
					continue;
				}
				open_first = r == 1;
			}
			else
			{
				if(!x.live) continue;
				passed = !ldcg(flags + f);
			}
			FieldState st = {};
			st.i = x.i;
			st.j = x.j;
			st.d = x.d;
			st.iter = x.iter;
			st.n_iter = x.n_iter;
			st.max_iter = x.max_iter;
			st.n_limits = x.nl;
			st.win_s = x.win_s;
			st.win_e = x.win_e;
			st.relax = rx[q];
			if(streamed)
			{
				// limits through L2 (see prefetch_limits)
				if(!open_first) close_sweep(st, passed);
				open_sweep(a.fields[f], st, blockIdx.x == 0);
			}
			else
			{
				close_sweep(st, passed);
				open_sweep_cached(blockIdx.x == 0 ? a.fields + f : nullptr, st, x, passed);
			}
			x.i = st.i;
			x.j = st.j;
			x.d = st.d;
			x.iter = st.iter;
			x.n_iter = st.n_iter;
			x.live = STREAM ? (x.live & 0xFF000000u) | st.live : st.live;
			x.win_s = st.win_s;
			x.win_e = st.win_e;
			x.chk_e = st.chk_e;
			rx[q] = st.relax;
		}
		__syncthreads();
		if constexpr(STREAM)
			if(s_sj == step)
			{
				// every streamed field's toplesets are done, and every streamed field
				// is a plain field from this boundary on: the schedules go back to
				// the FieldState (below), and the plain kernel's launch that follows
				// sweeps the rest
				if(blockIdx.x == 0 && threadIdx.x == 0) a.bar[3] = step + 1;
				const uint32_t w = __reduce_add_sync(0xffffffffu, n_skip);
				if(lane == 0 && w) atomicAdd(reinterpret_cast<unsigned long long *>(a.bar + 4), (unsigned long long) w);
				break;
			}
		grid_plan<TV, STREAM>(fs, ts, G, &s_tile);
		for(uint32_t q = threadIdx.x; q < G; q += NT) prefetch_limits<STREAM>(a.fields[id[q]], fs[q]);
	}
	if(blockIdx.x == 0)
		for(uint32_t q = threadIdx.x; q < G; q += NT)
		{
			const SchedSmem &x = fs[q];
			FieldState &g = a.state[id[q]];
			g.i = x.i;
			g.j = x.j;
			g.d = x.d;
			g.iter = x.iter;
			g.n_iter = x.n_iter;
			g.relax = rx[q];
			// (streaming: the launch that resumes reads the open windows)
			g.live = STREAM ? x.live & 1u : 0u;
			if constexpr(STREAM)
			{
				g.max_iter = x.max_iter;
				g.n_limits = x.nl;
				g.win_s = x.win_s;
				g.win_e = x.win_e;
				g.chk_e = x.chk_e;
			}
		}
}

size_t grid_smem_bytes(uint32_t F)
{
	static_assert(sizeof(SchedSmem) % 4 == 0, "layout");
	return 8 * (size_t) F + sizeof(SchedSmem) * F + 4 * (size_t) (F + 1) + 4 * (size_t) F;
}

// ---------------------------------------------------------------------------
// Work-queue sweeps: the grid-wide sweeps without a grid-wide barrier.
//
// Fields are independent; sweep s+1 of a field needs only sweep s of the same
// field to be complete.  So every warp of one persistent launch claims tiles
// (32 * groups consecutive window vertices) of whichever field has work,
// relaxes them, and counts them done; the warp that completes a field's sweep
// applies the reference's schedule rule (close_sweep / open_sweep) to that
// field alone and publishes the next window.  A field's short sweeps no
// longer wait for every other field's long ones, and no warp waits at a
// barrier: tail latency of one window is filled with tiles of the others.
//
// Ordering: tile writes -> __syncwarp -> fence -> completion add; the warp
// that sees the last completion fences, updates the schedule, writes the next
// window (sched[epoch & 1]), fences and swaps the cursors.  A claim that
// returns (epoch, k < tiles) is valid, and its sched entry cannot change until
// that tile is counted done.  Distances are read with L2 loads (__ldcg).
// Idle warps poll with growing sleeps and give up (error bit + abort) only if
// no sweep of any field completes for QUEUE_IDLE_NS.
// ---------------------------------------------------------------------------
constexpr unsigned long long QUEUE_IDLE_NS = 2000000000ull;  // 2 s without any completed sweep
constexpr uint32_t QB = 26;
constexpr unsigned long long QMASK = (1ull << QB) - 1;
constexpr uint32_t QUEUE_MAX_GROUPS = 32;  // at most 1024 vertices per tile

__device__ __forceinline__ unsigned long long qpack(uint32_t epoch, uint32_t tiles)
{
	return ((unsigned long long) (epoch & 0xFFFu) << (2 * QB)) | ((unsigned long long) tiles << QB);
}
__device__ __forceinline__ uint32_t q_index(unsigned long long c) { return (uint32_t) (c & QMASK); }
__device__ __forceinline__ uint32_t q_tiles(unsigned long long c) { return (uint32_t) ((c >> QB) & QMASK); }
__device__ __forceinline__ uint32_t q_epoch(unsigned long long c) { return (uint32_t) (c >> (2 * QB)); }

struct QueueArgs {
	FieldDev *fields;
	FieldState *state;
	uint32_t n_fields;
	QField *qf;
	QLine *cur;    // G * QUEUE_STRIPES claim cursors
	QLine *done;   // G * QUEUE_STRIPES completion counters
	QLine *sdone;  // G completed-stripe counters
	QCtl *ctl;
};

// Tile geometry of a window of nw vertices: groups of 32 vertices per tile
// (req, or enough that a window has at most ~256 tiles: claims on one cursor
// are serialised in L2), tiles, and non-empty stripes.
__device__ __forceinline__ void q_geometry(uint32_t nw, uint32_t req, uint32_t &groups, uint32_t &tiles,
                                           uint32_t &stripes)
{
	groups = req ? req : min(QUEUE_MAX_GROUPS, max(1u, (nw + 32u * 256u - 1) / (32u * 256u)));
	tiles = max(1u, (nw + 32u * groups - 1) / (32u * groups));
	stripes = min(QUEUE_STRIPES, tiles);
}

// Publish sweep `epoch` of queued field q with window [win_s, win_e).
__device__ void q_publish(const QueueArgs &a, uint32_t q, uint32_t epoch, uint32_t win_s, uint32_t win_e,
                          uint32_t chk_e, uint32_t d, uint32_t req)
{
	uint32_t groups, tiles, stripes;
	q_geometry(win_e - win_s, req, groups, tiles, stripes);
	QField &Q = a.qf[q];
	Q.sched[epoch & 1u] = make_uint4(win_s, win_e, chk_e, d | (groups << 1));
	st_relaxed(&Q.notok[epoch & 1u], 0u);
	for(uint32_t z = 0; z < QUEUE_STRIPES; z++) st_relaxed(&a.done[q * QUEUE_STRIPES + z].w, 0ull);
	st_relaxed(&a.sdone[q].w, 0ull);
	__threadfence();
	for(uint32_t z = 0; z < QUEUE_STRIPES; z++)
	{
		const uint32_t n = z < stripes ? (z + 1) * tiles / stripes - z * tiles / stripes : 0u;
		atomicExch(&a.cur[q * QUEUE_STRIPES + z].w, qpack(epoch, n));
	}
}

// The sweep `epoch` of queued field q is complete: apply the schedule rule
// (run_ptp_gpu, src/cuda/geodesics_ptp.cu:206-229) and publish the next sweep,
// or retire the field.  One thread.
__device__ void q_finish(const QueueArgs &a, uint32_t q, uint32_t epoch, uint32_t req)
{
	QField &Q = a.qf[q];
	const uint32_t f = Q.f;
	const FieldDev &F = a.fields[f];
	const uint4 sc = __ldcg(&Q.sched[epoch & 1u]);
	FieldState st = {};
	st.i = ld_relaxed(&Q.i);
	st.j = ld_relaxed(&Q.j);
	st.d = ld_relaxed(&Q.d);
	st.iter = ld_relaxed(&Q.iter);
	st.n_iter = ld_relaxed(&Q.n_iter);
	st.max_iter = Q.max_iter;
	st.n_limits = Q.n_limits;
	st.win_s = sc.x;
	st.win_e = sc.y;
	st.relax = ld_relaxed(&Q.relax);
	close_sweep(st, !ld_relaxed(&Q.notok[epoch & 1u]));
	open_sweep(F, st, true);
	st_relaxed(&Q.i, st.i);
	st_relaxed(&Q.j, st.j);
	st_relaxed(&Q.d, st.d);
	st_relaxed(&Q.iter, st.iter);
	st_relaxed(&Q.n_iter, st.n_iter);
	st_relaxed(&Q.relax, st.relax);
	if(st.live) q_publish(a, q, epoch + 1, st.win_s, st.win_e, st.chk_e, st.d, req);
	else
	{
		FieldState &g = a.state[f];
		g.i = st.i;
		g.j = st.j;
		g.d = st.d;
		g.iter = st.iter;
		g.n_iter = st.n_iter;
		g.relax = st.relax;
		g.live = 0;
		__threadfence();
		atomicSub(&a.ctl->live, 1u);
	}
	atomicAdd(&a.ctl->progress, 1u);
}

// Compact the fields handed to the grid, choose the launch (mode_req:
// GRID_LOCKSTEP, GRID_QUEUE, or 0 = queue when at least min_queue fields) and
// publish every queued field's first sweep.  One CTA of 1024 threads.
__global__ void __launch_bounds__(1024) queue_setup_kernel(QueueArgs a, uint32_t mode_req, uint32_t min_queue,
                                                           uint32_t warps, uint32_t groups)
{
	__shared__ uint32_t s_G;
	if(threadIdx.x == 0) s_G = 0;
	__syncthreads();
	for(uint32_t base = 0; base < a.n_fields; base += 1024)
	{
		const uint32_t f = base + threadIdx.x;
		const bool on = f < a.n_fields && a.state[f].big && a.state[f].live;
		uint32_t tot;
		const uint32_t ex = block_exclusive_scan<1024>(on ? 1u : 0u, &tot);
		if(on)
		{
			const FieldState &g = a.state[f];
			QField &Q = a.qf[s_G + ex];
			Q.f = f;
			Q.n_limits = g.n_limits;
			Q.max_iter = g.max_iter;
			Q.i = g.i;
			Q.j = g.j;
			Q.d = g.d;
			Q.iter = g.iter;
			Q.n_iter = g.n_iter;
			Q.relax = g.relax;
		}
		__syncthreads();
		if(threadIdx.x == 0) s_G += tot;
		__syncthreads();
	}
	const uint32_t G = s_G;
	const uint32_t mode = !G ? GRID_NONE
	                          : mode_req == GRID_LOCKSTEP || (mode_req != GRID_QUEUE && G < min_queue) ? GRID_LOCKSTEP
	                                                                                                   : GRID_QUEUE;
	if(mode == GRID_QUEUE)
		for(uint32_t q = threadIdx.x; q < G; q += 1024)
		{
			const FieldState &g = a.state[a.qf[q].f];
			q_publish(a, q, 0, g.win_s, g.win_e, g.chk_e, g.d, groups);
		}
	if(threadIdx.x == 0)
	{
		a.ctl->G = G;
		a.ctl->mode = mode;
		a.ctl->live = mode == GRID_QUEUE ? G : 0u;
		a.ctl->progress = 0;
		a.ctl->abort = 0;
		a.ctl->err = 0;
		a.ctl->warps = warps;
		a.ctl->groups = groups;
	}
}

__device__ __forceinline__ void red_add_release(uint32_t *p, uint32_t v)
{
	asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// A warp holds at most one unprocessed claim besides the tile it works on:
// while it relaxes tile k it has already claimed the next tile of the same
// stripe (the claim's latency overlaps the work).  Completions of ordinary
// tiles are fire-and-forget adds; the warp that claimed a stripe's last tile
// holds no other claim, waits (bounded) until the stripe's other tiles are
// counted, and then closes the stripe, and the sweep if it was the last
// stripe.  Every wait is for warps that hold claims and never wait
// themselves while holding one, so the waits end.
template <typename T, bool CL>
__global__ void __launch_bounds__(NT, GP_GRID_MINB) ptp_queue_kernel(QueueArgs a)
{
	if(a.ctl->mode != GRID_QUEUE) return;
	const uint32_t lane = threadIdx.x & 31;
	const uint32_t req = a.ctl->groups;
	const uint32_t wid = blockIdx.x * (NT / 32) + (threadIdx.x >> 5);
	const uint32_t Z = a.ctl->G * QUEUE_STRIPES;
	// home slot: warps spread evenly over the fields' stripes; a warp looks
	// there first and scans onwards only when its home has no work
	const uint32_t home = wid % Z;
	uint32_t seen = 0xFFFFFFFFu, backoff = 32;
	unsigned long long idle_t0 = 0;
	uint32_t z = Z;              // slot of the claim in hand (Z: none)
	unsigned long long c = 0;    // the claim in hand
	for(;;)
	{
		if(z == Z)
		{
			// lanes read 32 cursors at once, lane 0 claims from the first that shows work
			for(uint32_t base = 0; base < Z && z == Z; base += 32)
			{
				const uint32_t zz = (home + base + lane) % Z;
				bool avail = false;
				if(base + lane < Z)
				{
					const unsigned long long cv = ld_relaxed(&a.cur[zz].w);
					avail = q_index(cv) < q_tiles(cv);
				}
				unsigned m = __ballot_sync(0xffffffffu, avail);
				while(m)
				{
					const int l = __ffs(m) - 1;
					m &= m - 1;
					const uint32_t zl = __shfl_sync(0xffffffffu, zz, l);
					unsigned long long got = 0;
					if(lane == 0) got = atom_add_acquire(&a.cur[zl].w, 1ull);
					got = __shfl_sync(0xffffffffu, got, 0);
					if(q_index(got) < q_tiles(got))
					{
						z = zl;
						c = got;
						break;
					}
				}
			}
			if(z == Z)
			{
				uint32_t stop = 0;
				if(lane == 0)
				{
					const uint32_t p = ld_relaxed(&a.ctl->progress);
					const unsigned long long now = global_ns();
					if(ld_relaxed(&a.ctl->live) == 0 || ld_relaxed(&a.ctl->abort)) stop = 1;
					else if(p != seen)
					{
						seen = p;
						idle_t0 = now;
					}
					else if(now - idle_t0 > QUEUE_IDLE_NS)
					{
						atomicOr(&a.ctl->err, DEV_ERR_TIMEOUT);
						atomicExch(&a.ctl->abort, 1u);
						stop = 1;
					}
				}
				if(__shfl_sync(0xffffffffu, stop, 0)) return;
				__nanosleep(backoff);
				backoff = min(backoff * 2, 2048u);
				continue;
			}
		}
		backoff = 32;
		const uint32_t q = z / QUEUE_STRIPES, zs = z % QUEUE_STRIPES, e = q_epoch(c);
		const bool last = q_index(c) + 1 == q_tiles(c);
		unsigned long long nxt = 0;
		if(!last && lane == 0) nxt = atom_add_acquire(&a.cur[z].w, 1ull);
		__syncwarp();
		const uint4 sc = __ldcg(&a.qf[q].sched[e & 1u]);
		const uint32_t win_s = sc.x, win_e = sc.y, chk_e = sc.z, d = sc.w & 1u;
		uint32_t groups, tiles, stripes;
		q_geometry(win_e - win_s, req, groups, tiles, stripes);
		const uint32_t tile = zs * tiles / stripes + q_index(c);
		const FieldDev &F = a.fields[a.qf[q].f];
		int bad = 0;
		for(uint32_t g = 0; g < groups; g++)
		{
			const uint32_t v = win_s + (tile * groups + g) * 32u + lane;
			if(v < win_e) bad |= sweep_vertex<T, CL, true>(F, d, v, win_s, chk_e);
		}
		if(__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(&a.qf[q].notok[e & 1u], 1u);
		__syncwarp();
		uint32_t *done = reinterpret_cast<uint32_t *>(&a.done[z].w);
		if(!last)
		{
			if(lane == 0) red_add_release(done, 1u);
			nxt = __shfl_sync(0xffffffffu, nxt, 0);
			if(q_index(nxt) < q_tiles(nxt)) c = nxt;
			else z = Z;
			continue;
		}
		uint32_t ok = 1;
		if(lane == 0)
		{
			const uint32_t want = q_tiles(c) - 1;
			unsigned long long t0 = 0;
			uint32_t polls = 0;
			while(ld_acquire(done) < want)
			{
				if((++polls & 63u) == 0)
				{
					const unsigned long long now = global_ns();
					if(!t0) t0 = now;
					else if(now - t0 > QUEUE_IDLE_NS || ld_relaxed(&a.ctl->abort))
					{
						atomicOr(&a.ctl->err, DEV_ERR_TIMEOUT);
						atomicExch(&a.ctl->abort, 1u);
						ok = 0;
						break;
					}
				}
			}
			if(ok)
			{
				const uint32_t o2 = atom_add_acq_rel(reinterpret_cast<uint32_t *>(&a.sdone[q].w), 1u);
				if(o2 + 1 == stripes) q_finish(a, q, e, req);
			}
		}
		if(!__shfl_sync(0xffffffffu, ok, 0)) return;
		z = Z;
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
	unsigned long long *amax = nullptr;  // gather only: null, or max |out| (bits) of the call, atomicMax'ed
	bool nmax = false;                   // gather only: reduce each field's largest finite output into state.nmax
	// renumbering: write the CSR fan offsets (FP64, or FP32 rows longer than
	// a fan8 row can hold); false: cnt is not computed and off not written
	bool csr = true;
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
		if(c.fields[f].stream) continue;  // renumbered inside the sweep launch
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
		const uint32_t nr = st.n_limits && !F.stream ? F.limits[st.n_limits - 1] : 0;
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
		if(F.stream) continue;  // renumbered inside the sweep launch
		const FieldState &st = c.state[f];
		const uint32_t nr = st.n_limits ? F.limits[st.n_limits - 1] : 0;
		const uint32_t n0 = st.n_limits >= 2 ? F.limits[1] : nr;
		// FP32 path: double-float (hi, lo) pairs; FP64 path: double
		using S = typename std::conditional<sizeof(T) == 4, float2, double>::type;
		S *D0 = static_cast<S *>(F.D[0]);
		S *D1 = static_cast<S *>(F.D[1]);
		if(k < nr)
		{
			const uint32_t v = F.sorted[k];
			const uint32_t o0f = F.m.fan_off[v];
			const uint32_t o0 = o0f & FAN_MASK, o1 = F.m.fan_off[v + 1] & FAN_MASK;
			const uint32_t dst = c.csr ? c.cnt[g] : 0u;
			if(c.csr) F.off[k] = dst | (o0f & FAN_CLOSED);
			{
				uint32_t r[8];
				const uint32_t n = o1 - o0;
				for(uint32_t q = 0; q < 8; q++)
				{
					uint32_t x = FAN8_EMPTY;
					if(q < n)
					{
						const uint32_t iu = F.inv[F.m.fan[o0 + q]];
						x = iu ? iu - 1 : nr;
					}
					r[q] = x;
				}
				// a row holds at most 8 entries, a closed one at most 7 (its first
				// neighbour is repeated after the last, see below); longer rows are
				// read from the renumbered CSR fan, which the FP64 sweeps always read
				const bool cl = (o0f & FAN_CLOSED) != 0;
				const bool ovf = n > 8 || (cl && n == 8);
				if(sizeof(T) == 8 || ovf)
					for(uint32_t e = o0; e < o1; e++)
					{
						const uint32_t q = e - o0;
						uint32_t x = q < 8 ? r[q] : 0u;
						if(q >= 8)
						{
							const uint32_t iu = F.inv[F.m.fan[e]];
							x = iu ? iu - 1 : nr;
						}
						F.fan[dst + q] = x;
					}
				// Padding: a closed fan repeats its first neighbour after its last
				// (so the closing triangle is one more consecutive pair), and the
				// slots after that repeat the row's last entry (pairs of one vertex,
				// which the lean sweeps recognise by their equal ids).  Every slot
				// of a row of 1-8 entries then names a real neighbour.
				if(n && !ovf)
				{
					const uint32_t pad = cl ? r[0] : r[n - 1];
					for(uint32_t q = n; q < 8; q++) r[q] = pad;
				}
				if(ovf) r[7] = FAN8_OVERFLOW;
				// the star keeps the reference's triangle order (che::link from
				// EVT), so the label rule's "first strictly smaller candidate"
				// picks the same triangle as the reference in exact ties.  Slot 0
				// packs closed | count | first neighbour (see FAN8_N_SHIFT)
				r[0] = n ? (r[0] & FAN8_ID_MASK) | ((ovf ? 0u : n) << FAN8_N_SHIFT) | (cl ? FAN_CLOSED : 0u) : 0u;
				F.fan8[2 * (size_t) k] = make_uint4(r[0], r[1], r[2], r[3]);
				F.fan8[2 * (size_t) k + 1] = make_uint4(r[4], r[5], r[6], r[7]);
			}
			F.P[k] = F.m.pos[v];
			if(F.Pd)
			{
				const float4 pf = F.m.pos[v];
				F.Pd[4 * (size_t) k] = F.round_coords ? (double) pf.x : F.m.posd[4 * (size_t) v];
				F.Pd[4 * (size_t) k + 1] = F.round_coords ? (double) pf.y : F.m.posd[4 * (size_t) v + 1];
				F.Pd[4 * (size_t) k + 2] = F.round_coords ? (double) pf.z : F.m.posd[4 * (size_t) v + 2];
				F.Pd[4 * (size_t) k + 3] = 0.0;
			}
			S d0;
			// FP32: every vertex but the sources starts flagged as changed
			if constexpr(sizeof(T) == 4) d0 = make_float2(k < n0 ? 0.f : -INFINITY, 0.f);
			else d0 = k < n0 ? 0.0 : (double) INFINITY;
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
			if(c.csr) F.off[k] = c.cnt[g];
			F.fan8[2 * (size_t) k] = make_uint4(0u, FAN8_EMPTY, FAN8_EMPTY, FAN8_EMPTY);  // count 0
			F.fan8[2 * (size_t) k + 1] = make_uint4(FAN8_EMPTY, FAN8_EMPTY, FAN8_EMPTY, FAN8_EMPTY);
			F.P[k] = make_float4(0.f, 0.f, 0.f, 0.f);
			if(F.Pd)
				for(int q = 0; q < 4; q++) F.Pd[4 * (size_t) k + q] = 0.0;
			if constexpr(sizeof(T) == 4)
			{
				D0[k] = make_float2(INFINITY, 0.f);
				D1[k] = make_float2(INFINITY, 0.f);
			}
			else
			{
				D0[k] = (double) INFINITY;
				D1[k] = (double) INFINITY;
			}
			if(CL) { F.C[0][k] = 0; F.C[1][k] = 0; }
		}
	}
}

template <typename T, bool CL>
__global__ void gather_kernel(CatArgs c)
{
	unsigned long long mloc = 0;
	for(uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < c.total; g += gridDim.x * blockDim.x)
	{
		const uint32_t f = upper_index(c.base, c.n_fields, g);
		const uint32_t v = g - c.base[f];
		const FieldDev &F = c.fields[f];
		if(v >= F.m.nv) continue;
		const FieldState &st = c.state[f];
		const uint32_t iv = F.inv[v];
		const uint32_t k = iv ? iv - 1 : st.nr;
		// y: the value written (as a double, for the maxima below)
		double y;
		if constexpr(sizeof(T) == 4)
		{
			const float2 h = unflag(static_cast<const float2 *>(F.D[st.d])[k]);
			if(F.out_f64) static_cast<double *>(F.dist_out)[v] = y = (double) h.x + (double) h.y;
			else
			{
				// the float nearest hi + lo: one float addition (the double sum of a
				// normalized pair, at most 49 significant bits, is exact, so rounding
				// it to float gives the same bits); no FP64 work per vertex
				const float r = __fadd_rn(h.x, h.y);
				static_cast<float *>(F.dist_out)[v] = r;
				y = r;
			}
		}
		else
		{
			const double x = static_cast<const double *>(F.D[st.d])[k];
			if(F.out_f64) static_cast<double *>(F.dist_out)[v] = y = x;
			else static_cast<float *>(F.dist_out)[v] = (float) x, y = (double) (float) x;
		}
		if(CL && F.clusters_out)
			F.clusters_out[v] = iv ? F.C[st.d][k] : (F.clusters_in ? F.clusters_in[v] : 0u);
		// farthest-point sampling: max |out| over the call (the value cublasI?amax
		// looks for, src/cuda/geodesics_ptp.cu:138-142), fused into the gather
		if(c.amax) mloc = max(mloc, (unsigned long long) __double_as_longlong(fabs(y)));
		if(c.nmax)
		{
			// normalize_ptp's maximum over dist[v] < INFINITY (distances are >= 0,
			// so the bit patterns order like the values): lanes of one field
			// reduce together, 32-bit halves at a time, and one of them adds it
			const unsigned long long b = y < INFINITY && y > 0 ? (unsigned long long) __double_as_longlong(y) : 0ull;
			const unsigned grp = __match_any_sync(__activemask(), f);
			const uint32_t hi = __reduce_max_sync(grp, (uint32_t) (b >> 32));
			const uint32_t lo = __reduce_max_sync(grp, (uint32_t) (b >> 32) == hi ? (uint32_t) b : 0u);
			if((threadIdx.x & 31) == (uint32_t) (__ffs(grp) - 1) && hi)
				atomicMax(&c.state[f].nmax, ((unsigned long long) hi << 32) | lo);
		}
	}
	if(c.amax)
	{
		for(int o = 16; o; o >>= 1) mloc = max(mloc, __shfl_xor_sync(0xffffffffu, mloc, o));
		if((threadIdx.x & 31) == 0 && mloc) atomicMax(c.amax, mloc);
	}
}

// normalize_ptp (src/geodesics_ptp.cpp:264-276) of every field's output, on
// the maximum the gather reduced: dist[v] /= max_d.
template <typename O>
__global__ void normalize_batch_kernel(CatArgs c)
{
	for(uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < c.total; g += gridDim.x * blockDim.x)
	{
		const uint32_t f = upper_index(c.base, c.n_fields, g);
		const uint32_t v = g - c.base[f];
		const FieldDev &F = c.fields[f];
		if(v >= F.m.nv) continue;
		const O m = (O) __longlong_as_double((long long) c.state[f].nmax);
		static_cast<O *>(F.dist_out)[v] /= m;
	}
}

// ---------------------------------------------------------------------------
// Farthest-point sampling on the device (farthest_point_sampling_ptp_gpu,
// src/cuda/geodesics_ptp.cu:122-147): the sample loop runs without a host
// round trip.  Per sample: fps_sources_kernel sets the field's source count
// from the device counter, the usual BFS / renumbering / sweeps / gather run
// (the gather also reduces max |d|), fps_first_kernel finds the first vertex
// holding that maximum (cublasI?amax's pick, 0-based) and fps_append_kernel
// appends it and applies the loop's stop rule.  Once stopped, later samples change nothing.
// ---------------------------------------------------------------------------
__global__ void fps_sources_kernel(FieldDev *field, const FpsDev *c)
{
	if(threadIdx.x == 0) field->ns = c->ns;
}

// The first vertex whose |d| is the maximum the gather found (grid-wide:
// every thread checks its vertices, the smallest index wins).
template <typename T>
__global__ void fps_first_kernel(const T *x, uint32_t n, FpsDev *c)
{
	const unsigned long long m = c->amax;
	uint32_t best = 0xFFFFFFFFu;
	for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
		if((unsigned long long) __double_as_longlong(fabs((double) x[i])) == m)
		{
			best = i;
			break;
		}
	best = __reduce_min_sync(0xffffffffu, best);
	if((threadIdx.x & 31) == 0 && best != 0xFFFFFFFFu) atomicMin(&c->first, best);
}

__global__ void fps_append_kernel(FpsDev *c, uint32_t *samples, double radio, FpsErr e)
{
	if(threadIdx.x != 0) return;
	const unsigned long long m = c->amax;
	const uint32_t first = c->first;
	c->amax = 0;  // for the next sample
	c->first = 0xFFFFFFFFu;
	// this sample's device errors (they are cleared before the next sample runs)
	uint32_t err = e.sync[0].err | e.sync[1].err | e.bar[2] | e.ctl->err | e.state->status;
	if(e.wbar) err |= e.wbar[2];
	if(err)
	{
		c->err |= err;
		c->stop = 1;
	}
	if(c->stop || first == 0xFFFFFFFFu) return;
	samples[c->ns] = first;
	c->ns++;
	const double md = __longlong_as_double((long long) m);
	c->max_dist = md;
	// while(n-- && max_dist > radio): with a radius the loop ends once it is
	// reached (without one the reference never reads max_dist before the end)
	if((radio > 0 && !(md > radio)) || c->ns >= c->ns_max) c->stop = 1;
}

// ---------------------------------------------------------------------------
// normalize_ptp of a caller array (gp_normalize_ptp)
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

unsigned grid_for(uint64_t n)
{
	return (unsigned) std::max<uint64_t>(1, std::min<uint64_t>((n + 255) / 256, 152ull * 32));
}

} // namespace

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------

// csr: the FP32 sweeps read the CSR fan only for rows of more than a fan8
// row's entries, so a call whose meshes have none skips the counts, their
// scan and the offsets (csr false); FP64 always writes them.  inv_ready: the
// GPU toplesets already wrote inv (positions + 1, 0 for unreached vertices);
// host-given toplesets need it built here.
cudaError_t launch_renumber_batch(FieldDev *fields, FieldState *state, const uint32_t *base, uint32_t n_fields,
                                  uint32_t total, uint32_t *cnt, uint32_t *scan_tmp, bool f64, bool clusters,
                                  bool csr, bool inv_ready, cudaStream_t s)
{
	CatArgs c{fields, state, base, n_fields, total, cnt};
	c.csr = csr || f64;
	const unsigned nb = grid_for(total);
	if(!inv_ready)
	{
		inv_clear_kernel<<<nb, 256, 0, s>>>(c);
		inv_set_kernel<<<nb, 256, 0, s>>>(c);
	}
	if(c.csr)
	{
		count_kernel<<<nb, 256, 0, s>>>(c);
		const cudaError_t e = launch_scan_u32(cnt, cnt, total, scan_tmp, s);
		if(e != cudaSuccess) return e;
	}
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

cudaError_t launch_fps_sources(FieldDev *field, const FpsDev *c, cudaStream_t s)
{
	fps_sources_kernel<<<1, 32, 0, s>>>(field, c);
	return cudaGetLastError();
}

cudaError_t launch_fps_append(const void *dist, bool f64, uint32_t n, FpsDev *c, uint32_t *samples, double radio,
                              const FpsErr &e, cudaStream_t s)
{
	const unsigned nb = grid_for(n);
	if(f64) fps_first_kernel<double><<<nb, 256, 0, s>>>((const double *) dist, n, c);
	else fps_first_kernel<float><<<nb, 256, 0, s>>>((const float *) dist, n, c);
	fps_append_kernel<<<1, 32, 0, s>>>(c, samples, radio, e);
	return cudaGetLastError();
}

cudaError_t launch_normalize_batch(FieldDev *fields, FieldState *state, const uint32_t *base, uint32_t n_fields,
                                   uint32_t total, bool out_f64, cudaStream_t s)
{
	CatArgs c{fields, state, base, n_fields, total, nullptr};
	const unsigned nb = grid_for(total);
	if(out_f64) normalize_batch_kernel<double><<<nb, 256, 0, s>>>(c);
	else normalize_batch_kernel<float><<<nb, 256, 0, s>>>(c);
	return cudaGetLastError();
}

cudaError_t launch_gather_batch(FieldDev *fields, FieldState *state, const uint32_t *base, uint32_t n_fields,
                                uint32_t total, bool f64, bool clusters, cudaStream_t s, unsigned long long *amax,
                                bool nmax)
{
	CatArgs c{fields, state, base, n_fields, total, nullptr, amax, nmax};
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

static const void *ptp_kernel_ptr(bool f64, bool clusters, bool stream = false)
{
	if(f64)
		return clusters ? (const void *) ptp_kernel<double, true, false> : (const void *) ptp_kernel<double, false, false>;
	if(clusters) return (const void *) ptp_kernel<float, true, false>;
	return stream ? (const void *) ptp_kernel<float, false, true> : (const void *) ptp_kernel<float, false, false>;
}

// grid launches keep the schedules of up to this many fields in shared memory
constexpr uint32_t GRID_MAX_FIELDS = 2048;

// CTAs of a grid launch over n_fields fields: every SM's share at the shared
// memory this launch really uses (the schedule copy grows with n_fields).
int ptp_max_ctas(int device, bool f64, bool clusters, uint32_t n_fields)
{
	int nsm = 0, per = 0;
	cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
	const void *k = ptp_kernel_ptr(f64, clusters);
	cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) grid_smem_bytes(GRID_MAX_FIELDS));
	if(!f64 && !clusters)
		cudaFuncSetAttribute(ptp_kernel_ptr(false, false, true), cudaFuncAttributeMaxDynamicSharedMemorySize,
		                     (int) grid_smem_bytes(GRID_MAX_FIELDS));
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, NT, grid_smem_bytes(std::max<uint32_t>(n_fields, 1)));
	return nsm * per;
}

static const void *ptp_queue_ptr(bool f64, bool clusters)
{
	if(f64)
		return clusters ? (const void *) ptp_queue_kernel<double, true> : (const void *) ptp_queue_kernel<double, false>;
	return clusters ? (const void *) ptp_queue_kernel<float, true> : (const void *) ptp_queue_kernel<float, false>;
}

int ptp_queue_max_ctas(int device, bool f64, bool clusters)
{
	int nsm = 0, per = 0;
	cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, ptp_queue_ptr(f64, clusters), NT, 0);
	return nsm * per;
}

// Queue setup (which also makes the lockstep/queue choice) and the queue
// launch; the lockstep launch follows it and runs only if it was chosen.
cudaError_t launch_ptp_queue(FieldDev *fields, FieldState *state, uint32_t n_fields, QField *qf, QLine *cur,
                             QLine *done, QLine *sdone, QCtl *ctl, uint32_t ctas, uint32_t mode_req,
                             uint32_t min_queue, uint32_t tile, bool f64, bool clusters, cudaStream_t s)
{
	if(!n_fields) return cudaSuccess;
	QueueArgs a{fields, state, n_fields, qf, cur, done, sdone, ctl};
	ctas = std::max<uint32_t>(ctas, 1u);
	queue_setup_kernel<<<1, 1024, 0, s>>>(a, mode_req, min_queue, ctas * (NT / 32), std::min(tile / 32u, QUEUE_MAX_GROUPS));
	cudaError_t e = cudaGetLastError();
	if(e != cudaSuccess) return e;
	void *args[] = {&a};
	return cudaLaunchKernel(ptp_queue_ptr(f64, clusters), dim3(ctas), dim3(NT), args, 0, s);
}


uint32_t ptp_grid_max_fields() { return GRID_MAX_FIELDS; }

// binaryVersion of the FP32 sweep kernel's loaded code on the current device
int ptp_binary_version()
{
	cudaFuncAttributes a{};
	if(cudaFuncGetAttributes(&a, ptp_kernel_ptr(false, false)) != cudaSuccess)
	{
		cudaGetLastError();
		return 0;
	}
	return a.binaryVersion;
}

// notok: 3 * n_fields words; bar: 4 words.  Both zeroed here.
cudaError_t launch_ptp(FieldDev *fields, FieldState *state, uint32_t n_fields, uint32_t *notok, uint32_t *bar,
                       uint32_t ctas, bool f64, bool clusters, unsigned long long *steps, uint32_t steps_cap,
                       const QCtl *ctl, uint32_t spin_limit, uint32_t phantom, const uint32_t *sids,
                       uint32_t n_stream, uint32_t workers, unsigned long long *sprog, unsigned long long *snap,
                       cudaStream_t s)
{
	if(!n_fields) return cudaSuccess;
	if(n_stream && (f64 || clusters || n_stream > STREAM_MAX || !workers || workers >= ctas ||
	                n_stream > workers * STREAM_PER_WORKER))
		return cudaErrorInvalidValue;
	cudaError_t e = cudaMemsetAsync(notok, 0, 3 * sizeof(uint32_t) * n_fields, s);
	if(e == cudaSuccess) e = cudaMemsetAsync(bar, 0, GRID_BAR_WORDS * sizeof(uint32_t), s);
	if(e == cudaSuccess && steps) e = cudaMemsetAsync(steps, 0, 16 * (size_t) steps_cap, s);
	if(e == cudaSuccess && n_stream) e = cudaMemsetAsync(sprog, 0, sizeof(unsigned long long) * n_stream, s);
	if(e == cudaSuccess && n_stream)
		e = cudaMemsetAsync(snap + SNAP_DONE, 0, sizeof(unsigned long long) * SNAP_CTL_WORDS, s);
	if(e != cudaSuccess) return e;
	const uint32_t w = n_stream ? workers : 0u;
	GridArgs a{fields,  state, n_fields, notok, bar,      steps, steps_cap, ctl, spin_limit ? spin_limit : SPIN_LIMIT,
	           phantom, sids,  n_stream, w,     ctas - w, sprog, snap,     nullptr};
	void *args[] = {&a};
	e = cudaLaunchCooperativeKernel(ptp_kernel_ptr(f64, clusters, n_stream != 0), dim3(ctas), dim3(NT), args,
	                                grid_smem_bytes(n_fields), s);
	if(e != cudaSuccess || !n_stream) return e;
	// the streaming launch ends once every streamed field's toplesets are done;
	// the plain kernel sweeps the rest from the FieldState, on the second half
	// of the barrier line and with fresh ring-test flags
	e = cudaMemsetAsync(notok, 0, 3 * sizeof(uint32_t) * n_fields, s);
	if(e != cudaSuccess) return e;
	GridArgs b{fields,  state, n_fields, notok,   bar + BAR_RESUME, steps,   steps_cap, ctl, a.spin_limit,
	           phantom, sids,  0u,       0u,      ctas,             nullptr, nullptr,   bar};
	void *bargs[] = {&b};
	return cudaLaunchCooperativeKernel(ptp_kernel_ptr(f64, clusters, false), dim3(ctas), dim3(NT), bargs,
	                                   grid_smem_bytes(n_fields), s);
}

// 64-bit words of GridArgs::snap (progress snapshots and the done counts)
size_t ptp_snap_words(uint32_t)
{
	return SNAP_WORDS;
}

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
                            const uint32_t *pred_big, cudaStream_t s)
{
	if(!n_fields) return cudaSuccess;
	classify_kernel<<<(n_fields * 32 + 255) / 256, 256, 0, s>>>(fields, state, n_fields, local_window, pred_big);
	return cudaGetLastError();
}

// queue: one word, zeroed here (the field ticket); perm: null or the order
// in which fields are taken
cudaError_t launch_ptp_local(FieldDev *fields, FieldState *state, uint32_t n_fields, uint32_t *queue,
                             uint32_t ctas, uint32_t local_window, const uint32_t *perm, bool f64, bool clusters,
                             cudaStream_t s)
{
	cudaError_t e = cudaMemsetAsync(queue, 0, sizeof(uint32_t), s);
	if(e != cudaSuccess) return e;
	ctas = std::max<uint32_t>(1, std::min<uint32_t>(ctas, n_fields));
	void *args[] = {&fields, &state, &n_fields, &queue, &local_window, &perm};
	return cudaLaunchKernel(ptp_local_ptr(f64, clusters), dim3(ctas), dim3(LT), args, 0, s);
}

cudaError_t launch_field_features(const FieldDev *fields, const FieldState *state, uint32_t n_fields, float *out,
                                  cudaStream_t s)
{
	if(!n_fields) return cudaSuccess;
	field_features_kernel<<<(n_fields * 32 + 255) / 256, 256, 0, s>>>(fields, state, n_fields, out);
	return cudaGetLastError();
}

cudaError_t launch_plan(const FieldDev *fields, const FieldState *state, uint32_t n_fields, const float *pred,
                        uint32_t local_window, uint32_t *pred_big, float *cost, uint32_t *perm, cudaStream_t s)
{
	if(!n_fields) return cudaSuccess;
	plan_kernel<<<1, 1024, 0, s>>>(fields, state, n_fields, pred, local_window, LT, pred_big, cost, perm);
	return cudaGetLastError();
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

} // namespace gp
