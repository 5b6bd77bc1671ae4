/*
 * CPU oracle for gproshan's Parallel Toplesets Propagation (PTP) geodesics.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm used to check the CUDA path (tests, the smoke check) and timed as
 * the CPU baseline by bench.py.  The product path never links or calls it.
 *
 * Every function names the reference file:line it restates.  The FP64
 * arithmetic follows the reference operation by operation so that, compiled
 * with -ffp-contract=off, results equal the reference's own compiled code bit
 * for bit (checked by tests against the reference build and committed golden
 * vectors).
 */
#ifndef GP_PTP_ORACLE_H
#define GP_PTP_ORACLE_H

#include <stdint.h>

#define ORC_NIL 0xFFFFFFFFu
#define ORC_PTP_TOL 1e-3

#ifdef __cplusplus
extern "C" {
#endif

/* che::update_evt_ot_et (src/che.cpp:1295-1362): opposite table OT[3*nf] and
 * extra vertex table EVT[nv] from VT[3*nf].  Returns 1 if the mesh is
 * manifold, 0 otherwise (some EVT entries set to NIL), -1 on bad input. */
int orc_che_build(uint32_t nv, uint32_t nf, const uint32_t *VT, uint32_t *OT, uint32_t *EVT);

/* che::compute_toplesets + che::link (src/che.cpp:546-593, 102-112).
 * rings[nv]; sorted[cap_sorted]; limits[cap_limits].  Returns the number of
 * limits written (0 if there are no sources or a buffer is too small). */
uint32_t orc_toplesets(uint32_t nv, uint32_t nhe, const uint32_t *VT, const uint32_t *OT,
                       const uint32_t *EVT, const uint32_t *src, uint32_t n_src,
                       uint32_t *rings, uint32_t *sorted, uint32_t cap_sorted,
                       uint32_t *limits, uint32_t cap_limits);

/* update_step (src/geodesics_ptp.cpp:201-262), FP64. xyz is n_v*3 doubles. */
double orc_update_step(const double *xyz, const uint32_t *VT, const double *dist, uint32_t he);

/* Result of one PTP solve. */
typedef struct {
	uint32_t n_iter;      /* relaxation sweeps run */
	uint32_t last;        /* which buffer the last sweep wrote (0 or 1) */
	uint64_t relaxations; /* vertex relaxations performed (sum of window sizes) */
} orc_ptp_info;

/*
 * PTP with the schedule of run_ptp_gpu (src/cuda/geodesics_ptp.cu:174-232),
 * which is also the schedule of the CPU twins (src/geodesics_ptp.cpp:122-199),
 * in FP64 on the original vertex numbering.
 *
 * buf0/buf1 (nv each) receive the two Jacobi buffers; buf[info.last] is what
 * the GPU entry points return, buf[!info.last] is what the CPU entry points
 * return (they copy pdist[!d] after the final flip).
 * clusters0/clusters1 may be null; if given, they hold the initial labels
 * (non-source entries are taken as they are, as run_ptp_gpu does) and receive
 * the GPU labelling rule (src/cuda/geodesics_ptp.cu:257-282).
 * trace (may be null) receives (i, j) per sweep, 2*trace_cap entries at most.
 * nthreads <= 0 uses the OpenMP default.
 */
orc_ptp_info orc_ptp(uint32_t nv, const double *xyz, const uint32_t *VT, const uint32_t *OT,
                     const uint32_t *EVT, const uint32_t *src, uint32_t n_src,
                     const uint32_t *limits, uint32_t n_limits, const uint32_t *sorted,
                     double *buf0, double *buf1, uint32_t *clusters0, uint32_t *clusters1,
                     uint32_t *trace, uint32_t trace_cap, int nthreads);

/*
 * Same sweep as orc_ptp, but the schedule (i, j) per sweep is given instead of
 * decided by the convergence test.  Used to separate arithmetic error from
 * schedule divergence when comparing a reduced-precision run.
 */
orc_ptp_info orc_ptp_replay(uint32_t nv, const double *xyz, const uint32_t *VT, const uint32_t *OT,
                            const uint32_t *EVT, const uint32_t *src, uint32_t n_src,
                            const uint32_t *limits, uint32_t n_limits, const uint32_t *sorted,
                            const uint32_t *trace, uint32_t n_trace,
                            double *buf0, double *buf1, int nthreads);

/* normalize_ptp (src/geodesics_ptp.cpp:264-276). */
void orc_normalize_ptp(double *dist, uint64_t n);

/*
 * farthest_point_sampling_ptp_gpu (src/cuda/geodesics_ptp.cu:87-172):
 * samples holds n_init seeds on entry and up to cap entries on return.
 * Returns the number of samples; *max_dist receives the returned radius.
 */
uint32_t orc_fps(uint32_t nv, const double *xyz, const uint32_t *VT, const uint32_t *OT,
                 const uint32_t *EVT, uint32_t *samples, uint32_t n_init, uint32_t cap,
                 uint64_t n, double radio, double *max_dist, int nthreads);

#ifdef __cplusplus
}
#endif

#endif /* GP_PTP_ORACLE_H */
