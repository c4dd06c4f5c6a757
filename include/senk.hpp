/**
 * @file senk.hpp
 * @brief Top-level header of the GB300 build of SenK's solver path: the same
 * macros and includes as the reference's include/senk.hpp, with the solvers,
 * sparse kernels and blas1 running on the GPU (link libsenk_gpu.so); the
 * MatrixMarket reader (senk_io.hpp) and the setup functions are host code.
 */
#ifndef SENK_HPP
#define SENK_HPP

#define PRINT_RES false
#define ITER_SYMBOL "I"
#define TIME_SYMBOL "T"
#define RES_SYMBOL "#"

#include "senk_io.hpp"
#include "senk_matrix.hpp"
#include "senk_utils.hpp"
#include "senk_graph.hpp"
#include "senk_bicgstab.hpp"
#include "senk_gmres.hpp"
#include "senk_gcr.hpp"

/**
 * @namespace senk
 * @brief The top-level namespace of SenK.
 */

#endif
