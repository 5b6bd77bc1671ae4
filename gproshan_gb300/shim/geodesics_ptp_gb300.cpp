// Drop-in replacement for gproshan's GPU PTP entry points
// (src/cuda/geodesics_ptp.cu and src/cuda/geodesics_ptp_coalescence.cu),
// implemented over libgp_ptp.so's C ABI (include/gp_ptp.h).
//
// A gproshan build that compiles this file instead of those two .cu files and
// links libgp_ptp.so keeps the declarations of include/geodesics_ptp.h:34-42
// and the geodesics::PTP_GPU dispatch (src/geodesics.cpp:225-240) unchanged.
// Differences from the reference, all deliberate:
//   * no cudaDeviceReset (the reference resets the device on every call,
//     src/cuda/geodesics_ptp.cu:22); one gp_ctx per host thread is kept, and
//     made again when another part of the application has reset the device
//     since (gproshan's heat-flow entry points do, src/cuda/heat_flow.cu:47);
//   * errors are reported (gproshan_error + INFINITY distances) instead of
//     being ignored;
//   * distance_t may be double (default build) or float (SINGLE_P): the
//     library writes either type directly.  A double build computes in FP64
//     by default (the reference formula, bit-exact with the reference's
//     arithmetic); the environment variable GP_PTP_PRECISION=f32 makes it
//     compute in FP32 instead (within 1e-5 of FP64; about 50x faster on
//     GB300, whose FP64 pipe is narrow), still writing doubles.
#include <cstdlib>
#include <cstring>
#include "geodesics_ptp.h"

#include "gp_ptp.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

namespace gproshan {

namespace {

gp_ctx *thread_ctx()
{
	thread_local struct holder {
		gp_ctx *ctx = nullptr;
		~holder() { gp_ctx_destroy(ctx); }
	} h;
	if(h.ctx && !gp_ctx_valid(h.ctx))
	{
		// the device was reset since: the context's handles are gone
		gp_ctx_destroy(h.ctx);
		h.ctx = nullptr;
	}
	if(!h.ctx && gp_ctx_create(0, &h.ctx) != GP_OK) h.ctx = nullptr;
	return h.ctx;
}

constexpr gp_dtype dist_type = sizeof(distance_t) == sizeof(double) ? GP_F64 : GP_F32;

// Arithmetic of the solve: distance_t's, unless GP_PTP_PRECISION says
// otherwise ("f32" or "f64"); read once per process.
uint32_t precision()
{
	static const uint32_t p = [] {
		const char *e = std::getenv("GP_PTP_PRECISION");
		if(e && !std::strcmp(e, "f32")) return (uint32_t) GP_F32;
		if(e && !std::strcmp(e, "f64")) return (uint32_t) GP_F64;
		return (uint32_t) dist_type;
	}();
	return p;
}

// Upload the che (GT/VT/OT/EVT, as cuda_create_CHE does, src/cuda/che.cu:29-48).
gp_mesh *upload(gp_ctx *ctx, che *mesh)
{
	const size_t nv = mesh->n_vertices(), nhe = mesh->n_half_edges();
	std::vector<double> xyz(3 * nv);
	for(index_t v = 0; v < nv; v++)
		for(index_t k = 0; k < 3; k++) xyz[3 * v + k] = (double) mesh->gt(v)[k];
	std::vector<uint32_t> VT(nhe), OT(nhe), EVT(nv);
	for(index_t he = 0; he < nhe; he++)
	{
		VT[he] = mesh->vt(he);
		OT[he] = mesh->ot(he);
	}
	for(index_t v = 0; v < nv; v++) EVT[v] = mesh->evt(v);
	gp_mesh *m = nullptr;
	if(gp_mesh_create(ctx, (uint32_t) nv, xyz.data(), (uint32_t) mesh->n_faces(), VT.data(), OT.data(), EVT.data(),
	                  &m) != GP_OK)
		return nullptr;
	return m;
}

double run(const ptp_out_t &ptp_out, che *mesh, const std::vector<index_t> &sources, const toplesets_t &toplesets)
{
	gp_ctx *ctx = thread_ctx();
	gp_mesh *m = ctx ? upload(ctx, mesh) : nullptr;
	gp_ptp_stats stats{};
	gp_ptp_opts opts{};
	opts.precision = precision();  // FP64 builds run the reference formula in FP64 unless told otherwise
	gp_status st = GP_ERR_NO_DEVICE;
	if(m)
		st = gp_ptp(ctx, m, sources.data(), (uint32_t) sources.size(), toplesets.limits.data(),
		            (uint32_t) toplesets.limits.size(), toplesets.index, &opts, ptp_out.dist, dist_type,
		            ptp_out.clusters, &stats);
	gp_mesh_destroy(m);
	if(st != GP_OK)
	{
		fprintf(stderr, "[ERROR] gp_ptp: %s (%s)\n", gp_status_str(st), ctx ? gp_ctx_last_error(ctx) : "");
		for(index_t v = 0; v < mesh->n_vertices(); v++) ptp_out.dist[v] = INFINITY;
		return 0;
	}
	return stats.seconds;
}

} // namespace

double parallel_toplesets_propagation_gpu(const ptp_out_t &ptp_out, che *mesh, const std::vector<index_t> &sources,
                                          const toplesets_t &toplesets)
{
	return run(ptp_out, mesh, sources, toplesets);
}

double parallel_toplesets_propagation_coalescence_gpu(const ptp_out_t &ptp_out, che *mesh,
                                                      const std::vector<index_t> &sources,
                                                      const toplesets_t &toplesets, const bool &)
{
	// The library always sweeps a ring-renumbered copy, so the solve is the
	// same call.  What differs is the output rule of this entry point
	// (src/cuda/geodesics_ptp_coalescence.cu:62-86): only the vertices the
	// toplesets reached (toplesets.index[0, limits.back())) are written; every
	// other vertex keeps the caller's distance and label.
	const size_t nv = mesh->n_vertices();
	const index_t nr = toplesets.limits.empty() ? 0 : toplesets.limits.back();
	std::vector<distance_t> dist(nv);
	std::vector<index_t> lab(ptp_out.clusters ? nv : 0);
	if(ptp_out.clusters) std::copy(ptp_out.clusters, ptp_out.clusters + nv, lab.begin());
	const double t = run(ptp_out_t(dist.data(), ptp_out.clusters ? lab.data() : nullptr), mesh, sources, toplesets);
	for(index_t i = 0; i < nr; i++)
	{
		const index_t v = toplesets.index[i];
		ptp_out.dist[v] = dist[v];
		if(ptp_out.clusters) ptp_out.clusters[v] = lab[v];
	}
	return t;
}

distance_t farthest_point_sampling_ptp_gpu(che *mesh, std::vector<index_t> &samples, double &time_fps, size_t n,
                                           distance_t radio)
{
	gp_ctx *ctx = thread_ctx();
	gp_mesh *m = ctx ? upload(ctx, mesh) : nullptr;
	if(samples.empty()) samples.push_back(0);
	const size_t cap = std::max(n, samples.size()) + 1;
	std::vector<uint32_t> s(cap);
	for(size_t k = 0; k < samples.size(); k++) s[k] = samples[k];
	uint32_t n_out = 0;
	double md = INFINITY, sec = 0;
	gp_ptp_opts opts{};
	opts.precision = precision();
	const gp_status st = m ? gp_fps(ctx, m, s.data(), (uint32_t) samples.size(), (uint32_t) cap, n, radio, &opts,
	                                &n_out, &md, &sec)
	                       : GP_ERR_NO_DEVICE;
	gp_mesh_destroy(m);
	time_fps = sec;
	if(st != GP_OK)
	{
		fprintf(stderr, "[ERROR] gp_fps: %s\n", gp_status_str(st));
		return INFINITY;
	}
	samples.assign(s.begin(), s.begin() + n_out);
	return (distance_t) md;
}

} // namespace gproshan
