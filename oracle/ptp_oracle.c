/*
 * CPU oracle for gproshan's PTP geodesics -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference algorithm.  Tests compare the CUDA
 * path against it, the smoke check uses it as the checker, and bench.py times
 * it as the CPU baseline ("port").  Nothing in the product path loads it.
 *
 * Half-edge conventions follow the reference's compact half-edge mesh (CHE):
 * triangle t owns half-edges 3t, 3t+1, 3t+2; VT[he] is the origin vertex of
 * he; OT[he] is the opposite half-edge or NIL; EVT[v] is one outgoing
 * half-edge of v (include/che.h:41-47).
 */
#include "ptp_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define NIL ORC_NIL

/* trig/next/prev (src/che.cpp:18-34) */
static inline uint32_t he_next(uint32_t he) { return he == NIL ? NIL : 3 * (he / 3) + (he + 1) % 3; }
static inline uint32_t he_prev(uint32_t he) { return he == NIL ? NIL : 3 * (he / 3) + (he + 2) % 3; }

int orc_che_build(uint32_t nv, uint32_t nf, const uint32_t *VT, uint32_t *OT, uint32_t *EVT)
{
	/* che::update_evt_ot_et, src/che.cpp:1295-1362 */
	const uint64_t nhe = 3ull * nf;
	int manifold = 1;
	for(uint32_t v = 0; v < nv; v++) EVT[v] = NIL;
	if(!nf) return 1;
	for(uint64_t he = 0; he < nhe; he++)
		if(VT[he] >= nv) return -1;

	/* half-edges per origin vertex, in increasing half-edge order (CSR) */
	uint32_t *cnt = calloc((size_t) nv + 1, sizeof(uint32_t));
	uint32_t *lst = malloc(sizeof(uint32_t) * (nhe ? nhe : 1));
	for(uint64_t he = 0; he < nhe; he++)
	{
		EVT[VT[he]] = (uint32_t) he;
		cnt[VT[he] + 1]++;
	}
	for(uint32_t v = 0; v < nv; v++) cnt[v + 1] += cnt[v];
	uint32_t *fill = malloc(sizeof(uint32_t) * ((size_t) nv + 1));
	memcpy(fill, cnt, sizeof(uint32_t) * ((size_t) nv + 1));
	for(uint64_t he = 0; he < nhe; he++)
		lst[fill[VT[he]]++] = (uint32_t) he;

	for(uint64_t he = 0; he < nhe; he++) OT[he] = NIL;
	for(uint64_t he = 0; he < nhe; he++)
	{
		if(OT[he] != NIL) continue;
		const uint32_t a = VT[he];
		const uint32_t b = VT[he_next((uint32_t) he)];
		for(uint32_t k = cnt[a]; k < cnt[a + 1]; k++)
		{
			const uint32_t h = lst[k];
			const uint32_t ph = he_prev(h);
			if(VT[ph] == b && OT[he] == NIL && OT[ph] == NIL)
			{
				OT[he] = ph;
				OT[ph] = (uint32_t) he;
			}
		}
	}

	for(uint64_t he = 0; he < nhe; he++)
	{
		const uint32_t v = VT[he];
		if(OT[he] == NIL && EVT[v] != NIL)
		{
			if(OT[EVT[v]] == NIL && EVT[v] != he)
			{
				manifold = 0;
				EVT[v] = NIL;
			}
			else EVT[v] = (uint32_t) he;
		}
	}

	free(cnt);
	free(lst);
	free(fill);
	return manifold;
}

uint32_t orc_toplesets(uint32_t nv, uint32_t nhe, const uint32_t *VT, const uint32_t *OT,
                       const uint32_t *EVT, const uint32_t *src, uint32_t n_src,
                       uint32_t *rings, uint32_t *sorted, uint32_t cap_sorted,
                       uint32_t *limits, uint32_t cap_limits)
{
	/* che::compute_toplesets, src/che.cpp:546-593; che::link, src/che.cpp:102-112 */
	(void) nhe;
	if(!n_src || cap_limits < 2) return 0;
	for(uint32_t v = 0; v < nv; v++) rings[v] = NIL;

	uint32_t level = 0, p = 0, nl = 0;
	for(uint32_t s = 0; s < n_src; s++)
	{
		if(src[s] >= nv || p >= cap_sorted) return 0;
		sorted[p++] = src[s];
		if(rings[src[s]] == NIL) rings[src[s]] = level;
	}

	limits[nl++] = 0;
	for(uint32_t i = 0; i < p; i++)
	{
		const uint32_t v = sorted[i];
		if(rings[v] > level)
		{
			level++;
			if(nl >= cap_limits) return 0;
			limits[nl++] = i;
		}

		const uint32_t stop = EVT[v];
		for(uint32_t he = stop; he != NIL; )
		{
			uint32_t u = VT[he_next(he)];
			if(rings[u] == NIL)
			{
				if(p >= cap_sorted) return 0;
				rings[u] = rings[v] + 1;
				sorted[p++] = u;
			}
			if(OT[he_prev(he)] == NIL)
			{
				u = VT[he_prev(he)];
				if(rings[u] == NIL)
				{
					if(p >= cap_sorted) return 0;
					rings[u] = rings[v] + 1;
					sorted[p++] = u;
				}
			}
			he = OT[he_prev(he)];
			if(he == stop) he = NIL;
		}
	}

	if(nl >= cap_limits) return 0;
	limits[nl++] = p;
	return nl;
}

double orc_update_step(const double *xyz, const uint32_t *VT, const double *dist, uint32_t he)
{
	/* update_step, src/geodesics_ptp.cpp:201-262 (operation order kept) */
	uint32_t x[3];
	x[0] = VT[he_next(he)];
	x[1] = VT[he_prev(he)];
	x[2] = VT[he];

	const double *g0 = xyz + 3 * (size_t) x[0];
	const double *g1 = xyz + 3 * (size_t) x[1];
	const double *g2 = xyz + 3 * (size_t) x[2];
	double X[2][3];
	for(int k = 0; k < 3; k++)
	{
		X[0][k] = g0[k] - g2[k];
		X[1][k] = g1[k] - g2[k];
	}

	double t[2];
	t[0] = dist[x[0]];
	t[1] = dist[x[1]];

	double q[2][2];
	q[0][0] = X[0][0] * X[0][0] + X[0][1] * X[0][1] + X[0][2] * X[0][2];
	q[0][1] = X[0][0] * X[1][0] + X[0][1] * X[1][1] + X[0][2] * X[1][2];
	q[1][0] = X[1][0] * X[0][0] + X[1][1] * X[0][1] + X[1][2] * X[0][2];
	q[1][1] = X[1][0] * X[1][0] + X[1][1] * X[1][1] + X[1][2] * X[1][2];

	double det = q[0][0] * q[1][1] - q[0][1] * q[1][0];
	double Q[2][2];
	Q[0][0] = q[1][1] / det;
	Q[0][1] = -q[0][1] / det;
	Q[1][0] = -q[1][0] / det;
	Q[1][1] = q[0][0] / det;

	double delta = t[0] * (Q[0][0] + Q[1][0]) + t[1] * (Q[0][1] + Q[1][1]);
	double dis = delta * delta -
	             (Q[0][0] + Q[0][1] + Q[1][0] + Q[1][1]) *
	             (t[0] * t[0] * Q[0][0] + t[0] * t[1] * (Q[1][0] + Q[0][1]) + t[1] * t[1] * Q[1][1] - 1);

	double p = (delta + sqrt(dis)) / (Q[0][0] + Q[0][1] + Q[1][0] + Q[1][1]);

	double tp[2];
	tp[0] = t[0] - p;
	tp[1] = t[1] - p;

	double n[3];
	for(int k = 0; k < 3; k++)
		n[k] = tp[0] * (X[0][k] * Q[0][0] + X[1][k] * Q[1][0]) + tp[1] * (X[0][k] * Q[0][1] + X[1][k] * Q[1][1]);

	double cond[2];
	cond[0] = X[0][0] * n[0] + X[0][1] * n[1] + X[0][2] * n[2];
	cond[1] = X[1][0] * n[0] + X[1][1] * n[1] + X[1][2] * n[2];

	double c[2];
	c[0] = cond[0] * Q[0][0] + cond[1] * Q[0][1];
	c[1] = cond[0] * Q[1][0] + cond[1] * Q[1][1];

	if(t[0] == INFINITY || t[1] == INFINITY || dis < 0 || c[0] >= 0 || c[1] >= 0)
	{
		double dp[2];
		dp[0] = dist[x[0]] + sqrt(X[0][0] * X[0][0] + X[0][1] * X[0][1] + X[0][2] * X[0][2]);
		dp[1] = dist[x[1]] + sqrt(X[1][0] * X[1][0] + X[1][1] * X[1][1] + X[1][2] * X[1][2]);
		p = dp[dp[1] < dp[0]];
	}

	return p;
}

/* One Jacobi sweep over window [start, end) of sorted: relax_ptp
 * (src/cuda/geodesics_ptp.cu:234-282), same as the CPU loop body
 * (src/geodesics_ptp.cpp:205-223) but with the GPU cluster rule. */
static void sweep(const double *xyz, const uint32_t *VT, const uint32_t *OT, const uint32_t *EVT,
                  const uint32_t *sorted, uint32_t start, uint32_t end, uint32_t nv,
                  double *nd, const double *od, uint32_t *nc, const uint32_t *oc)
{
	#pragma omp parallel for schedule(static)
	for(int64_t vi = start; vi < (int64_t) end; vi++)
	{
		const uint32_t v = sorted[vi];
		if(v >= nv) continue;
		double best = od[v];
		uint32_t lab = oc ? oc[v] : 0;
		const uint32_t stop = EVT[v];
		for(uint32_t he = stop; he != NIL; )
		{
			const double d = orc_update_step(xyz, VT, od, he);
			if(d < best)
			{
				best = d;
				if(oc)
				{
					const uint32_t a = VT[he_prev(he)], b = VT[he_next(he)];
					lab = od[a] < od[b] ? oc[a] : oc[b];
				}
			}
			he = OT[he_prev(he)];
			if(he == stop) he = NIL;
		}
		nd[v] = best;
		if(nc) nc[v] = lab;
	}
}

/* relative_error + count_if(is_ok) (src/cuda/geodesics_ptp.cu:221-225, 284-299, 371-375) */
static int ring_converged(const uint32_t *sorted, uint32_t start, uint32_t n_cond,
                          const double *nd, const double *od)
{
	uint32_t count = 0;
	for(uint32_t vi = start; vi < start + n_cond; vi++)
	{
		const uint32_t v = sorted[vi];
		const double err = fabs(nd[v] - od[v]) / od[v];
		count += err < ORC_PTP_TOL;
	}
	return count == n_cond;
}

static void init_buffers(uint32_t nv, const uint32_t *src, uint32_t n_src, double *b0, double *b1,
                         uint32_t *c0, uint32_t *c1)
{
	for(uint32_t v = 0; v < nv; v++) b0[v] = b1[v] = INFINITY;
	for(uint32_t s = 0; s < n_src; s++) b0[src[s]] = b1[src[s]] = 0;
	if(c0)
	{
		for(uint32_t s = 0; s < n_src; s++) c0[src[s]] = s + 1;
		if(c1) memcpy(c1, c0, sizeof(uint32_t) * nv);
	}
}

orc_ptp_info orc_ptp(uint32_t nv, const double *xyz, const uint32_t *VT, const uint32_t *OT,
                     const uint32_t *EVT, const uint32_t *src, uint32_t n_src,
                     const uint32_t *limits, uint32_t n_limits, const uint32_t *sorted,
                     double *buf0, double *buf1, uint32_t *clusters0, uint32_t *clusters1,
                     uint32_t *trace, uint32_t trace_cap, int nthreads)
{
	/* run_ptp_gpu, src/cuda/geodesics_ptp.cu:174-232 */
#ifdef _OPENMP
	int saved = omp_get_max_threads();
	if(nthreads > 0) omp_set_num_threads(nthreads);
#else
	(void) nthreads;
#endif
	orc_ptp_info info = {0, 0, 0};
	double *buf[2] = {buf0, buf1};
	uint32_t *cl[2] = {clusters0, clusters1};
	init_buffers(nv, src, n_src, buf0, buf1, clusters0, clusters1);

	/* With fewer than three limits the reference reads past the end of
	 * limits (undefined behaviour); no sweep is run here. */
	if(n_limits >= 3)
	{
		uint32_t d = 0, i = 1, j = 2, iter = 0;
		const uint32_t max_iter = n_limits << 1;
		while(i < j && iter++ < max_iter)
		{
			if(i < (j >> 1)) i = j >> 1;
			const uint32_t start = limits[i], end = limits[j];
			const uint32_t n_cond = limits[i + 1] - start;
			if(trace && info.n_iter < trace_cap)
			{
				trace[2 * info.n_iter] = i;
				trace[2 * info.n_iter + 1] = j;
			}
			sweep(xyz, VT, OT, EVT, sorted, start, end, nv, buf[!d], buf[d],
			      clusters0 ? cl[!d] : NULL, clusters0 ? cl[d] : NULL);
			info.relaxations += end - start;
			if(ring_converged(sorted, start, n_cond, buf[!d], buf[d])) i++;
			if(j < n_limits - 1) j++;
			d = !d;
			info.n_iter++;
		}
		info.last = d;
	}
#ifdef _OPENMP
	omp_set_num_threads(saved);
#endif
	return info;
}

orc_ptp_info orc_ptp_replay(uint32_t nv, const double *xyz, const uint32_t *VT, const uint32_t *OT,
                            const uint32_t *EVT, const uint32_t *src, uint32_t n_src,
                            const uint32_t *limits, uint32_t n_limits, const uint32_t *sorted,
                            const uint32_t *trace, uint32_t n_trace,
                            double *buf0, double *buf1, int nthreads)
{
#ifdef _OPENMP
	int saved = omp_get_max_threads();
	if(nthreads > 0) omp_set_num_threads(nthreads);
#else
	(void) nthreads;
#endif
	orc_ptp_info info = {0, 0, 0};
	double *buf[2] = {buf0, buf1};
	init_buffers(nv, src, n_src, buf0, buf1, NULL, NULL);
	uint32_t d = 0;
	for(uint32_t t = 0; t < n_trace; t++)
	{
		const uint32_t i = trace[2 * t], j = trace[2 * t + 1];
		if(i >= n_limits || j >= n_limits || i > j) break;
		sweep(xyz, VT, OT, EVT, sorted, limits[i], limits[j], nv, buf[!d], buf[d], NULL, NULL);
		info.relaxations += limits[j] - limits[i];
		d = !d;
		info.n_iter++;
	}
	info.last = d;
#ifdef _OPENMP
	omp_set_num_threads(saved);
#endif
	return info;
}

void orc_normalize_ptp(double *dist, uint64_t n)
{
	/* normalize_ptp, src/geodesics_ptp.cpp:264-276 */
	double max_d = 0;
	for(uint64_t v = 0; v < n; v++)
		if(dist[v] < INFINITY && dist[v] > max_d) max_d = dist[v];
	for(uint64_t v = 0; v < n; v++)
		dist[v] /= max_d;
}

uint32_t orc_fps(uint32_t nv, const double *xyz, const uint32_t *VT, const uint32_t *OT,
                 const uint32_t *EVT, uint32_t *samples, uint32_t n_init, uint32_t cap,
                 uint64_t n, double radio, double *max_dist, int nthreads)
{
	/* farthest_point_sampling_ptp_gpu, src/cuda/geodesics_ptp.cu:87-172 */
	uint32_t ns = n_init;
	const uint32_t nhe = 0;
	uint32_t *rings = malloc(sizeof(uint32_t) * nv);
	uint32_t *sorted = malloc(sizeof(uint32_t) * ((size_t) nv + cap));
	uint32_t *limits = malloc(sizeof(uint32_t) * ((size_t) nv + 2));
	double *b0 = malloc(sizeof(double) * nv);
	double *b1 = malloc(sizeof(double) * nv);
	double md = INFINITY;

	if(n >= nv) n = nv >> 1;
	n = n > ns ? n - ns : 0; /* the reference underflows here when n < samples */

	while(n-- && md > radio && ns < cap)
	{
		uint32_t nl = orc_toplesets(nv, nhe, VT, OT, EVT, samples, ns, rings, sorted, nv + cap,
		                            limits, nv + 2);
		orc_ptp_info info = orc_ptp(nv, xyz, VT, OT, EVT, samples, ns, limits, nl, sorted,
		                            b0, b1, NULL, NULL, NULL, 0, nthreads);
		const double *dist = info.last ? b1 : b0;
		/* cublasI?amax: first index of the largest |x| */
		uint32_t f = 0;
		double best = -1;
		for(uint32_t v = 0; v < nv; v++)
		{
			const double a = fabs(dist[v]);
			if(a > best) { best = a; f = v; }
		}
		if(radio > 0 || !n) md = dist[f];
		samples[ns++] = f;
	}

	free(rings); free(sorted); free(limits); free(b0); free(b1);
	*max_dist = md;
	return ns;
}
