/*
 * Stand-in for the reference's include_arma.h, used only to compile the
 * reference's own mesh code (che.cpp) as the test oracle without Armadillo.
 *
 * The only Armadillo user in che.cpp is che::find_corr, which is not on the
 * geodesics path.  The types below make that function compile; every
 * operation aborts if it is ever reached at run time.
 */
#ifndef GP_ORACLE_STUB_INCLUDE_ARMA_H
#define GP_ORACLE_STUB_INCLUDE_ARMA_H

#include "include.h"

#include <cstdio>
#include <cstdlib>

namespace arma {

[[noreturn]] inline void stub_unreachable()
{
	std::fprintf(stderr, "oracle stub: Armadillo is not available in the oracle build\n");
	std::abort();
}

namespace fill { struct ones_t {}; constexpr ones_t ones{}; }
namespace solve_opts { struct no_approx_t {}; constexpr no_approx_t no_approx{}; }

template <class T>
struct stub_mat
{
	T cell{};
	stub_mat() = default;
	stub_mat(int, int, fill::ones_t) { stub_unreachable(); }
	explicit stub_mat(int) { stub_unreachable(); }
	stub_mat(T *, int, bool, bool) { stub_unreachable(); }
	T & operator()(int) { stub_unreachable(); }
	T & operator()(int, int) { stub_unreachable(); }
	stub_mat head(int) const { stub_unreachable(); }
	stub_mat submat(int, int, int, int) const { stub_unreachable(); }
	stub_mat cols(int, int) const { stub_unreachable(); }
	stub_mat col(int) const { stub_unreachable(); }
	stub_mat operator*(const stub_mat &) const { stub_unreachable(); }
	stub_mat operator-(const stub_mat &) const { stub_unreachable(); }
	stub_mat operator>=(const T &) const { stub_unreachable(); }
};

template <class T> bool all(const stub_mat<T> &) { stub_unreachable(); }
template <class T> T sum(const stub_mat<T> &) { stub_unreachable(); }
template <class T> T norm(const stub_mat<T> &) { stub_unreachable(); }
template <class T> stub_mat<T> solve(const stub_mat<T> &, const stub_mat<T> &) { stub_unreachable(); }
template <class T> bool solve(stub_mat<T> &, const stub_mat<T> &, const stub_mat<T> &, solve_opts::no_approx_t) { stub_unreachable(); }

typedef stub_mat<double> mat;
typedef stub_mat<double> vec;
typedef stub_mat<float> fmat;
typedef stub_mat<float> fvec;

} // namespace arma

namespace gproshan {

#ifdef SINGLE_P
	typedef arma::fmat a_mat;
	typedef arma::fvec a_vec;
#else
	typedef arma::mat a_mat;
	typedef arma::vec a_vec;
#endif

} // namespace gproshan

#endif // GP_ORACLE_STUB_INCLUDE_ARMA_H
