// Diagonal scaling of a CSR matrix in device memory: the reference's
// senk::matrix::GetDiag and Scaling (include/senk_matrix.hpp:391-416) and the
// symmetric scaling its driver applies before factorising (main.cpp:65-73,
// d_i = 1 / sqrt|a_ii|, a_ij <- d_i a_ij d_j).
//
// GetDiag: one thread per row scans the row for its diagonal (the first entry
// whose column is the row). Scaling: a group of kLanesPerRow lanes per row
// strides over the row's entries, so the groups of a warp read contiguous
// stretches of val and cind. Each value is (ld[i] * a_ij) * rd[j], products
// rounded separately in that order, and the factors 1 / sqrt|a_ii| use IEEE
// square root and division, so the results equal the host functions' bit for
// bit.
#include "device.hpp"

namespace senkgpu {

namespace {

constexpr int kLanesPerRow = 8;

__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double inv_sqrt_abs(double a) { return __ddiv_rn(1.0, __dsqrt_rn(fabs(a))); }
__device__ __forceinline__ float inv_sqrt_abs(float a) { return __fdiv_rn(1.0f, __fsqrt_rn(fabsf(a))); }

// diag[i] = a_ii (0 for a row without a diagonal entry); with INV, 1 / sqrt|a_ii|.
template <typename T, bool INV>
__global__ void __launch_bounds__(kThreads)
k_get_diag(const T *__restrict__ val, const int *__restrict__ cind, const int *__restrict__ rptr, T *__restrict__ diag,
           int N)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < N;
         i += (long long)gridDim.x * blockDim.x) {
        T d = T(0);
        const int e = rptr[i + 1];
        for (int j = rptr[i]; j < e; j++)
            if (cind[j] == (int)i) {
                d = val[j];
                break;
            }
        diag[i] = INV ? inv_sqrt_abs(d) : d;
    }
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
k_scaling(T *__restrict__ val, const int *__restrict__ cind, const int *__restrict__ rptr, const T *__restrict__ ld,
          const T *__restrict__ rd, int N)
{
    const long long groups = (long long)gridDim.x * blockDim.x / kLanesPerRow;
    const int lane = threadIdx.x % kLanesPerRow;
    for (long long i = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / kLanesPerRow; i < N; i += groups) {
        const T l = ld[i];
        const int e = rptr[i + 1];
        for (int j = rptr[i] + lane; j < e; j += kLanesPerRow) val[j] = mul_rn(mul_rn(l, val[j]), rd[cind[j]]);
    }
}

template <typename T>
int dev_get_diag(const T *val, const int *cind, const int *rptr, T *diag, int N, bool inv, cudaStream_t s)
{
    SENK_REQUIRE(val && cind && rptr && diag && N > 0, "null argument or empty matrix");
    const int grid = stream_grid(N, kThreads, 4);
    if (inv) k_get_diag<T, true><<<grid, kThreads, 0, s>>>(val, cind, rptr, diag, N);
    else k_get_diag<T, false><<<grid, kThreads, 0, s>>>(val, cind, rptr, diag, N);
    SENK_LAUNCH_CHECK();
    return (int)kOk;
}

template <typename T>
int dev_scaling(T *val, const int *cind, const int *rptr, const T *ld, const T *rd, int N, cudaStream_t s)
{
    SENK_REQUIRE(val && cind && rptr && ld && rd && N > 0, "null argument or empty matrix");
    const int grid = stream_grid((long long)N * kLanesPerRow, kThreads, 4);
    k_scaling<T><<<grid, kThreads, 0, s>>>(val, cind, rptr, ld, rd, N);
    SENK_LAUNCH_CHECK();
    return (int)kOk;
}

}  // namespace

}  // namespace senkgpu

using namespace senkgpu;

extern "C" {

int senk_dev_get_diag_d(const double *val, const int *cind, const int *rptr, double *diag, int N, void *stream)
{
    return guarded("senk_dev_get_diag_d",
                   [&] { return dev_get_diag<double>(val, cind, rptr, diag, N, false, (cudaStream_t)stream); });
}

int senk_dev_get_diag_s(const float *val, const int *cind, const int *rptr, float *diag, int N, void *stream)
{
    return guarded("senk_dev_get_diag_s",
                   [&] { return dev_get_diag<float>(val, cind, rptr, diag, N, false, (cudaStream_t)stream); });
}

int senk_dev_scaling_d(double *val, const int *cind, const int *rptr, const double *ld, const double *rd, int N,
                       void *stream)
{
    return guarded("senk_dev_scaling_d",
                   [&] { return dev_scaling<double>(val, cind, rptr, ld, rd, N, (cudaStream_t)stream); });
}

int senk_dev_scaling_s(float *val, const int *cind, const int *rptr, const float *ld, const float *rd, int N,
                       void *stream)
{
    return guarded("senk_dev_scaling_s",
                   [&] { return dev_scaling<float>(val, cind, rptr, ld, rd, N, (cudaStream_t)stream); });
}

int senk_dev_diag_scaling_d(double *val, const int *cind, const int *rptr, double *d, int N, void *stream)
{
    return guarded("senk_dev_diag_scaling_d", [&] {
        dev_get_diag<double>(val, cind, rptr, d, N, true, (cudaStream_t)stream);
        return dev_scaling<double>(val, cind, rptr, d, d, N, (cudaStream_t)stream);
    });
}

int senk_dev_diag_scaling_s(float *val, const int *cind, const int *rptr, float *d, int N, void *stream)
{
    return guarded("senk_dev_diag_scaling_s", [&] {
        dev_get_diag<float>(val, cind, rptr, d, N, true, (cudaStream_t)stream);
        return dev_scaling<float>(val, cind, rptr, d, d, N, (cudaStream_t)stream);
    });
}

}  // extern "C"
