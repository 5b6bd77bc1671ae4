// Test driver for the C++ drop-in (gproshan_gb300/shim/geodesics_ptp_gb300.cpp).
//
// Built by tests/test_dropin.py from the reference's own CPU sources (che,
// vertex, che_off, geodesics_ptp: the che class and the CPU PTP) plus the shim
// and libgp_ptp.so, it calls the reference's public GPU entry points the way
// gproshan's own callers do (src/geodesics.cpp:225-240, src/sampling.cpp:69)
// and writes the results as raw arrays for the Python side to compare with the
// oracle.  Test infrastructure only.
//
//   dropin <dir>   reads  <dir>/xyz.f64 (3 per vertex), <dir>/tri.u32 (3 per
//                  face), <dir>/src.u32 (sources), <dir>/fps.u32 (one word:
//                  samples to take)
//                  writes <dir>/gpu.dist, gpu_reset.dist (after a
//                  cudaDeviceReset), coal.dist, coal.cl, gpu.cl, fps_samples.u32,
//                  fps.max
//
// distance_t is double (the reference's default build) or float (-DSINGLE_P);
// .dist files hold distance_t values.
#include "che.h"
#include "geodesics_ptp.h"

#include <cuda_runtime.h>

#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

using namespace gproshan;

template <class T>
static std::vector<T> read_all(const std::string &path)
{
	std::ifstream f(path, std::ios::binary | std::ios::ate);
	if(!f) return {};
	const size_t n = (size_t) f.tellg() / sizeof(T);
	std::vector<T> v(n);
	f.seekg(0);
	f.read(reinterpret_cast<char *>(v.data()), (std::streamsize) (n * sizeof(T)));
	return v;
}

template <class T>
static void write_all(const std::string &path, const T *p, size_t n)
{
	std::ofstream f(path, std::ios::binary);
	f.write(reinterpret_cast<const char *>(p), (std::streamsize) (n * sizeof(T)));
}

int main(int argc, char **argv)
{
	if(argc != 2) return 2;
	const std::string dir = argv[1];
	const auto xyz = read_all<double>(dir + "/xyz.f64");
	const auto tri = read_all<unsigned>(dir + "/tri.u32");
	const auto src = read_all<unsigned>(dir + "/src.u32");
	const auto nfps = read_all<unsigned>(dir + "/fps.u32");
	if(xyz.empty() || tri.empty() || src.empty() || nfps.size() != 1) return 3;
	const size_t nv = xyz.size() / 3;
	std::vector<vertex> V(nv);
	for(size_t i = 0; i < nv; i++) V[i] = vertex((real_t) xyz[3 * i], (real_t) xyz[3 * i + 1], (real_t) xyz[3 * i + 2]);
	std::vector<index_t> F(tri.begin(), tri.end());
	che mesh(V.data(), nv, F.data(), F.size() / 3);

	const std::vector<index_t> sources(src.begin(), src.end());
	std::vector<index_t> rings(nv), sorted(nv + sources.size());
	std::vector<index_t> limits;
	index_t *r = rings.data(), *s = sorted.data();
	mesh.compute_toplesets(r, s, limits, sources);

	// parallel_toplesets_propagation_gpu, as geodesics::PTP_GPU calls it for several sources
	std::vector<distance_t> d(nv, 0);
	if(parallel_toplesets_propagation_gpu({d.data(), nullptr}, &mesh, sources, {limits, sorted.data()}) <= 0) return 4;
	write_all(dir + "/gpu.dist", d.data(), nv);

	// with labels (every label starts at 0; sources get 1-based indices)
	std::vector<index_t> cl(nv, 0);
	std::vector<distance_t> dl(nv, 0);
	parallel_toplesets_propagation_gpu({dl.data(), cl.data()}, &mesh, sources, {limits, sorted.data()});
	write_all(dir + "/gpu.cl", cl.data(), nv);

	// the coalescence entry point: unreached vertices keep the caller's values
	std::vector<distance_t> dc(nv, (distance_t) -7);
	std::vector<index_t> cc(nv, 12345);
	parallel_toplesets_propagation_coalescence_gpu({dc.data(), cc.data()}, &mesh, sources, {limits, sorted.data()});
	write_all(dir + "/coal.dist", dc.data(), nv);
	write_all(dir + "/coal.cl", cc.data(), nv);

	// another part of the application resets the device between calls
	// (gproshan's heat-flow entry points do): the next call still works
	if(cudaDeviceReset() != cudaSuccess) return 5;
	std::vector<distance_t> d2(nv, 0);
	parallel_toplesets_propagation_gpu({d2.data(), nullptr}, &mesh, sources, {limits, sorted.data()});
	write_all(dir + "/gpu_reset.dist", d2.data(), nv);

	// farthest-point sampling from vertex src[0]
	std::vector<index_t> samples = {sources[0]};
	double t_fps = 0;
	const distance_t md = farthest_point_sampling_ptp_gpu(&mesh, samples, t_fps, nfps[0], 0);
	write_all(dir + "/fps_samples.u32", samples.data(), samples.size());
	const double mdd = (double) md;
	write_all(dir + "/fps.max", &mdd, 1);
	return 0;
}
