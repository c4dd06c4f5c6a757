// Library-wide C ABI pieces: error reporting, version, device count, and the
// host setup functions (wrapping the drop-in headers in include/).
#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/senk_gpu.h"
#include "../../include/senk_graph.hpp"
#include "../../include/senk_io.hpp"
#include "../../include/senk_matrix.hpp"

namespace senkgpu {
namespace {
thread_local std::string g_last_error;
}
void set_last_error(const std::string &msg) { g_last_error = msg; }
}  // namespace senkgpu

using senkgpu::set_last_error;

extern "C" {

const char *senk_last_error(void) { return senkgpu::g_last_error.c_str(); }

int senk_version(void) { return 100; }

int senk_device_count(void)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

int senk_set_device(int device)
{
    const cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_last_error(std::string("senk_set_device: ") + cudaGetErrorString(e));
        return SENK_ERR_CUDA;
    }
    return SENK_OK;
}

void senk_free(void *p) { std::free(p); }

int senk_setup_ilu0(double *val, const int *cind, const int *rptr, int N)
{
    // The header's Ilu0 exits on a zero pivot (the reference's behaviour); the C
    // ABI reports it instead.
    const int row = senk::matrix::detail::ilu0(val, cind, rptr, N);
    if (row >= 0) {
        set_last_error("senk_setup_ilu0: zero pivot in row " + std::to_string(row));
        return SENK_ERR_ZERO_PIVOT;
    }
    return SENK_OK;
}

int senk_setup_split(const double *val, const int *cind, const int *rptr, double **lval, int **lcind,
                     int **lrptr, double **uval, int **ucind, int **urptr, double **diag, int N, const char *key,
                     int invDiag)
{
    if (!key || (std::strcmp(key, "LD-U") && std::strcmp(key, "L-DU") && std::strcmp(key, "L-D-U") &&
                 std::strcmp(key, "LU-D"))) {
        set_last_error("senk_setup_split: key must be LD-U, L-DU, L-D-U or LU-D");
        return SENK_ERR_ARG;
    }
    double *dummy = nullptr;
    senk::matrix::Split<double>(const_cast<double *>(val), const_cast<int *>(cind), const_cast<int *>(rptr), lval,
                                lcind, lrptr, uval, ucind, urptr, diag ? diag : &dummy, N, key, invDiag != 0);
    if (!diag && dummy) std::free(dummy);
    return SENK_OK;
}

int senk_setup_abmc_permutation(const int *cind, const int *rptr, int *num_color, int **size_color, int **LP,
                                int **RP, int N, int bsize, int isSym, const char *bmethod)
{
    if (bsize <= 0 || N % bsize) {
        set_last_error("senk_setup_abmc_permutation: N must be a multiple of bsize");
        return SENK_ERR_ARG;
    }
    if (!bmethod || (std::strcmp(bmethod, "simple") && std::strcmp(bmethod, "connect"))) {
        set_last_error("senk_setup_abmc_permutation: method must be simple or connect");
        return SENK_ERR_ARG;
    }
    senk::graph::GetABMCPermutation(const_cast<int *>(cind), const_cast<int *>(rptr), num_color, size_color, LP, RP,
                                    N, bsize, isSym != 0, bmethod);
    return SENK_OK;
}

int senk_setup_amc_permutation(const int *cind, const int *rptr, int *num_color, int **size_color, int **LP,
                               int **RP, int N, int isSym)
{
    senk::graph::GetAMCPermutation(const_cast<int *>(cind), const_cast<int *>(rptr), num_color, size_color, LP, RP,
                                   N, isSym != 0);
    return SENK_OK;
}

int senk_setup_reordering(double *val, int *cind, int *rptr, const int *LP, const int *RP, int N)
{
    senk::matrix::Reordering<double>(val, cind, rptr, const_cast<int *>(LP), const_cast<int *>(RP), N);
    return SENK_OK;
}

int senk_setup_csr2bcsr(const double *val, const int *cind, const int *rptr, double **bval, int **bcind,
                        int **brptr, int N, int bnl, int bnw)
{
    if (bnl <= 0 || bnw <= 0 || N % bnl || N % bnw) {
        set_last_error("senk_setup_csr2bcsr: N must be a multiple of bnl and bnw");
        return SENK_ERR_ARG;
    }
    senk::matrix::Csr2Bcsr<double>(const_cast<double *>(val), const_cast<int *>(cind), const_cast<int *>(rptr), bval,
                                   bcind, brptr, N, bnl, bnw);
    return SENK_OK;
}

int senk_io_read_matrix_market(const char *filename, double **val, int **cind, int **rptr, int *N, int *M,
                               int *symmetric, int remove_zeros)
{
    if (!filename || !val || !cind || !rptr || !N || !M || !symmetric) {
        set_last_error("senk_io_read_matrix_market: null argument");
        return SENK_ERR_ARG;
    }
    senk::io::Shape shape = senk::io::Unsym;
    if (!senk::io::ReadMatrixMarket(filename, val, cind, rptr, N, M, &shape, remove_zeros != 0)) {
        set_last_error(std::string("senk_io_read_matrix_market: cannot read ") + filename +
                       " (message on stderr)");
        return SENK_ERR_ARG;
    }
    *symmetric = shape == senk::io::Sym ? 1 : 0;
    return SENK_OK;
}

int senk_setup_expand(const double *tval, const int *tcind, const int *trptr, double **val, int **cind,
                      int **rptr, int N, const char *key)
{
    if (!key || (std::strcmp(key, "L") != 0 && std::strcmp(key, "U") != 0)) {
        set_last_error("senk_setup_expand: key must be \"L\" or \"U\"");
        return SENK_ERR_ARG;
    }
    senk::matrix::Expand<double>(const_cast<double *>(tval), const_cast<int *>(tcind), const_cast<int *>(trptr), val,
                                 cind, rptr, N, key);
    return SENK_OK;
}

int senk_setup_alloc_block_zero(double **val, int **cind, int **rptr, int N, int bnl, int bnw)
{
    if (bnl <= 0 || bnw <= 0 || N % bnl || N % bnw) {
        set_last_error("senk_setup_alloc_block_zero: N must be a multiple of bnl and bnw");
        return SENK_ERR_ARG;
    }
    senk::matrix::AllocBlockZero<double>(val, cind, rptr, N, bnl, bnw);
    return SENK_OK;
}

int senk_setup_ilup(double **val, int **cind, int **rptr, int N, int p)
{
    senk::matrix::Ilup<double>(val, cind, rptr, N, p);
    return SENK_OK;
}

int senk_setup_alloc_level_zero(double **val, int **cind, int **rptr, int N, int p)
{
    senk::matrix::AllocLevelZero<double>(val, cind, rptr, N, p);
    return SENK_OK;
}

int senk_setup_remove_off_diagonal(double **val, int **cind, int **rptr, int N, int bnum)
{
    if (!val || !cind || !rptr || N <= 0 || bnum <= 0 || N % bnum) {
        senkgpu::set_last_error("senk_setup_remove_off_diagonal: bad argument");
        return SENK_ERR_ARG;
    }
    senk::matrix::RemoveOffDiagonal<double>(val, cind, rptr, N, bnum);
    return SENK_OK;
}

}  // extern "C"
