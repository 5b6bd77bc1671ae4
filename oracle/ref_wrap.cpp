/*
 * Test-oracle shim over the reference's OWN CPU geodesics code.
 *
 * This file is test infrastructure.  It is compiled together with the
 * reference's src/che.cpp, src/vertex.cpp and src/geodesics_ptp.cpp, where
 * they lie, by oracle/Makefile into oracle/_ref/ (never committed), and is
 * loaded only by tests and by the fixture generator under tests/golden/.
 * It exposes a plain C ABI so Python can drive the unmodified reference:
 *
 *   - che(vertex*, n_v, faces, n_f)          include/che.h:53
 *   - che::compute_toplesets                src/che.cpp:546-593
 *   - parallel_toplesets_propagation_cpu    src/geodesics_ptp.cpp:122-199
 *   - parallel_toplesets_propagation_coalescence_cpu
 *                                           src/geodesics_ptp.cpp:40-120
 *   - update_step                           src/geodesics_ptp.cpp:201-262
 *   - normalize_ptp                         src/geodesics_ptp.cpp:264-276
 *   - geodesics(mesh, sources, PTP_CPU)     src/geodesics.cpp:16-33, 192-207
 *     (one field end to end: toplesets, then the coalescence CPU PTP)
 *   - che_off(file) (OFF reader)            src/che_off.cpp:28-79
 *
 * Built twice: once with real_t = double (the reference default) and once
 * with -DSINGLE_P (real_t = float).  The C entry points carry a suffix so
 * both libraries can be loaded into one process.  A third build (-DREF_GPU,
 * prefix refg_f64_) also links the reference's own GPU PTP
 * (src/cuda/geodesics_ptp.cu, geodesics_ptp_coalescence.cu, che.cu,
 * vertex.cu) and exposes geodesics_ptp_gpu; that path calls cudaDeviceReset on
 * every call, so it is only ever loaded by a process of its own.
 */
#include "che.h"
#include "che_off.h"
#include "geodesics_ptp.h"

#include <cmath>
#include <cstring>
#include <vector>

#if defined(REF_GPU)
#define REFW(name) refg_f64_##name
#elif defined(SINGLE_P)
#define REFW(name) refw_f32_##name
#else
#define REFW(name) refw_f64_##name
#endif

using gproshan::che;
using gproshan::index_t;
using gproshan::real_t;
using gproshan::distance_t;

extern "C" {

/* Build a reference che from xyz (double, n_v*3) and triangles (n_f*3). */
void * REFW(che_create)(const double * xyz, unsigned n_v, const unsigned * tri, unsigned n_f)
{
	std::vector<gproshan::vertex> V(n_v);
	for(unsigned i = 0; i < n_v; i++)
		V[i] = gproshan::vertex((real_t) xyz[3 * i], (real_t) xyz[3 * i + 1], (real_t) xyz[3 * i + 2]);
	std::vector<index_t> F(tri, tri + 3 * (size_t) n_f);
	return new che(V.data(), n_v, F.data(), n_f);
}

void REFW(che_free)(void * h)
{
	delete (che *) h;
}

/* Read an OFF file with the reference's reader (che_off). */
void * REFW(off_open)(const char * path)
{
	return new gproshan::che_off(path);
}

unsigned REFW(che_n_vertices)(void * h)
{
	return (unsigned) ((che *) h)->n_vertices();
}

/* Copy the coordinates (3 per vertex) out of the mesh. */
void REFW(che_xyz)(void * h, double * xyz)
{
	che * m = (che *) h;
	for(index_t v = 0; v < m->n_vertices(); v++)
	{
		const gproshan::vertex & p = m->gt(v);
		xyz[3 * v] = p.x;
		xyz[3 * v + 1] = p.y;
		xyz[3 * v + 2] = p.z;
	}
}

unsigned REFW(che_n_half_edges)(void * h)
{
	return (unsigned) ((che *) h)->n_half_edges();
}

/* Copy VT, OT (n_half_edges each) and EVT (n_vertices) out of the mesh. */
void REFW(che_tables)(void * h, unsigned * VT, unsigned * OT, unsigned * EVT)
{
	che * m = (che *) h;
	for(index_t he = 0; he < m->n_half_edges(); he++)
	{
		VT[he] = m->vt(he);
		OT[he] = m->ot(he);
	}
	for(index_t v = 0; v < m->n_vertices(); v++)
		EVT[v] = m->evt(v);
}

/*
 * che::compute_toplesets.  rings and sorted hold n_vertices entries (sorted
 * may need more when sources repeat: cap_sorted is its capacity), limits
 * holds cap_limits entries.  Returns the number of limits, or 0 when a
 * buffer is too small (nothing useful is written then).
 */
unsigned REFW(toplesets)(void * h, const unsigned * src, unsigned n_src,
                         unsigned * rings, unsigned * sorted, unsigned cap_sorted,
                         unsigned * limits, unsigned cap_limits)
{
	che * m = (che *) h;
	std::vector<index_t> sources(src, src + n_src);
	std::vector<index_t> lim;
	std::vector<index_t> srt(m->n_vertices() + n_src);
	index_t * r = rings;
	index_t * s = srt.data();
	m->compute_toplesets(r, s, lim, sources);
	if(lim.size() > cap_limits || lim.back() > cap_sorted) return 0;
	memcpy(limits, lim.data(), sizeof(index_t) * lim.size());
	memcpy(sorted, srt.data(), sizeof(index_t) * lim.back());
	return (unsigned) lim.size();
}

/*
 * Run the reference CPU PTP with caller-provided toplesets.
 * coalescence != 0 selects parallel_toplesets_propagation_coalescence_cpu
 * (what geodesics::PTP_CPU runs), otherwise parallel_toplesets_propagation_cpu.
 * clusters may be null.
 */
void REFW(ptp_cpu)(void * h, const unsigned * src, unsigned n_src,
                   const unsigned * limits, unsigned n_limits, const unsigned * sorted,
                   distance_t * dist, unsigned * clusters, int coalescence)
{
	che * m = (che *) h;
	std::vector<index_t> sources(src, src + n_src);
	std::vector<index_t> lim(limits, limits + n_limits);
	const index_t * idx = sorted;
	gproshan::toplesets_t ts = {lim, idx};
	gproshan::ptp_out_t out(dist, clusters);
	if(coalescence)
		gproshan::parallel_toplesets_propagation_coalescence_cpu(out, m, sources, ts);
	else
		gproshan::parallel_toplesets_propagation_cpu(out, m, sources, ts);
}

/*
 * One field the way geodesics(mesh, sources, PTP_CPU) computes it
 * (src/geodesics.cpp:16-33 and run_parallel_toplesets_propagation_cpu,
 * :192-207): dist set to INFINITY, che::compute_toplesets, then
 * parallel_toplesets_propagation_coalescence_cpu.  The timed unit of the
 * CPU baselines.  Returns the number of limits.
 */
unsigned REFW(geodesics_ptp_cpu)(void * h, const unsigned * src, unsigned n_src, distance_t * dist)
{
	che * m = (che *) h;
	const size_t n = m->n_vertices();
	for(size_t v = 0; v < n; v++)
		dist[v] = INFINITY;
	std::vector<index_t> sources(src, src + n_src);
	std::vector<index_t> toplesets(n), sorted(n + n_src), limits;
	index_t * r = toplesets.data();
	index_t * s = sorted.data();
	m->compute_toplesets(r, s, limits, sources);
	gproshan::parallel_toplesets_propagation_coalescence_cpu({dist, nullptr}, m, sources, {limits, s});
	return (unsigned) limits.size();
}

#ifdef REF_GPU
/*
 * One field the way geodesics(mesh, sources, PTP_GPU) computes it
 * (src/geodesics.cpp:16-33 and run_parallel_toplesets_propagation_gpu,
 * :225-240): dist set to INFINITY, che::compute_toplesets on the host, then
 * parallel_toplesets_propagation_coalescence_gpu for one source or
 * parallel_toplesets_propagation_gpu for several.  Returns the GPU seconds the
 * reference itself reports.
 */
double REFW(geodesics_ptp_gpu)(void * h, const unsigned * src, unsigned n_src, distance_t * dist)
{
	che * m = (che *) h;
	const size_t n = m->n_vertices();
	for(size_t v = 0; v < n; v++)
		dist[v] = INFINITY;
	std::vector<index_t> sources(src, src + n_src);
	std::vector<index_t> toplesets(n), sorted(n + n_src), limits;
	index_t * r = toplesets.data();
	index_t * s = sorted.data();
	m->compute_toplesets(r, s, limits, sources);
	if(sources.size() > 1)
		return gproshan::parallel_toplesets_propagation_gpu({dist, nullptr}, m, sources, {limits, s});
	return gproshan::parallel_toplesets_propagation_coalescence_gpu({dist, nullptr}, m, sources, {limits, s});
}
#endif

distance_t REFW(update_step)(void * h, const distance_t * dist, unsigned he)
{
	return gproshan::update_step((che *) h, dist, he);
}

void REFW(normalize_ptp)(distance_t * dist, unsigned long long n)
{
	gproshan::normalize_ptp(dist, (size_t) n);
}

int REFW(real_bytes)(void)
{
	return (int) sizeof(real_t);
}

} // extern "C"
