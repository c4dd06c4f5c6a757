/**
 * @file senk_test.hpp
 * @brief senk::test::RelativeResidualError (reference include/senk_test.hpp):
 * prints ‖b − A x‖ / ‖b‖, computed in FP64 on the GPU.
 */
#ifndef SENK_TEST_HPP
#define SENK_TEST_HPP

#include <cstdio>
#include <vector>

#include "senk_blas1.hpp"
#include "senk_sparse.hpp"

namespace senk {

namespace test {

inline void RelativeResidualError(double *val, int *cind, int *rptr, double *b, double *x, int N)
{
    std::vector<double> t(N);
    senk::sparse::SpmvCsr<double>(val, cind, rptr, x, t.data(), N);
    senk::blas1::Axpby<double>(1, b, -1, t.data(), N);
    const double nt = senk::blas1::Nrm2<double>(t.data(), N);
    const double nb = senk::blas1::Nrm2<double>(b, N);
    std::printf("# test %e\n", nt / nb);
}

}  // namespace test

}  // namespace senk

#endif
