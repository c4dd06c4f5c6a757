// ILU(0) numeric factorisation on the device (replaces the sequential
// senk::matrix::Ilu0, include/senk_matrix.hpp:418-448, for reordered systems).
//
// The reference eliminates row by row (IKJ): for row i and each of its lower
// entries k (ascending column c = cind[k] < i): val[k] /= u_cc, then every later
// entry j of row i whose column also appears in row c is updated,
// val[j] -= val[k] * val[l]. Row i only reads rows c < i of its lower pattern,
// which the schedule has finished: under an AMC/ABMC ordering they belong to an
// earlier colour or to the same chain (ABMC block), so the chains of a colour
// are factorised concurrently, one thread per chain, its rows in order; in the
// natural order the rows of one level set run concurrently. Every row performs
// the reference's operations in the reference's order with IEEE division and
// separately rounded products and differences (no FMA contraction), so the
// factors are the reference's bit for bit.
#include <algorithm>
#include <vector>

#include "device.hpp"

namespace senkgpu {

namespace {

__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }

// Chains [c0, c0 + nch) of one phase; chain t holds rows rows[(c0 + t) * bs + r],
// r < bs, factorised in that order.
template <typename T>
__global__ void __launch_bounds__(128)
k_ilu0_chains(T *val, const int *__restrict__ cind, const int *__restrict__ rptr, const int *__restrict__ rows,
              int c0, int nch, int bs, int *status)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nch) return;
    for (int r = 0; r < bs; r++) {
        const int i = rows[(long long)(c0 + t) * bs + r];
        if (i == 0) continue;  // the reference starts at row 1
        const int s = rptr[i], e = rptr[i + 1];
        for (int k = s; k < e; k++) {
            const int c = cind[k];
            if (c >= i) break;
            const int cs = rptr[c], ce = rptr[c + 1];
            for (int l = cs; l < ce; l++) {
                if (cind[l] == c) {
                    const T d = val[l];
                    if (d == T(0)) {
                        atomicExch(status, 1);
                        return;
                    }
                    val[k] = div_rn(val[k], d);
                    break;
                }
            }
            const T vk = val[k];
            int pos = cs;
            for (int j = k + 1; j < e; j++) {
                const int cj = cind[j];
                for (int l = pos; l < ce; l++) {
                    const int cl = cind[l];
                    if (cl < cj) continue;
                    pos = l;
                    if (cl == cj) {
                        val[j] = sub_rn(val[j], mul_rn(vk, val[l]));
                        pos++;
                    }
                    break;
                }
            }
        }
    }
}

// The schedule: rows in processing order and, per phase, a range of chains.
struct FactorSchedule {
    std::vector<int> rows;
    std::vector<int> phase_chains;  // chain ranges of the phases (size phases + 1)
    int bs = 1;
};

// Lower-pattern level sets (natural order): level(i) = 1 + max level of the
// rows i reads.
FactorSchedule level_sets(const std::vector<int> &cind, const std::vector<int> &rptr, int N)
{
    std::vector<int> lev(N, 0);
    int maxlev = 0;
    for (int i = 0; i < N; i++) {
        int l = 0;
        for (int j = rptr[i]; j < rptr[i + 1] && cind[j] < i; j++) l = std::max(l, lev[cind[j]] + 1);
        lev[i] = l;
        maxlev = std::max(maxlev, l);
    }
    std::vector<int> cnt(maxlev + 2, 0);
    for (int i = 0; i < N; i++) cnt[lev[i] + 1]++;
    for (int l = 0; l <= maxlev; l++) cnt[l + 1] += cnt[l];
    FactorSchedule f;
    f.rows.assign(N, 0);
    std::vector<int> at(cnt.begin(), cnt.end() - 1);
    for (int i = 0; i < N; i++) f.rows[at[lev[i]]++] = i;
    f.phase_chains = cnt;
    f.bs = 1;
    return f;
}

// Colours of chains (AMC: bs = 1). Checks that every lower column of a row is in
// an earlier colour or earlier in the row's own chain.
FactorSchedule colour_chains(const std::vector<int> &cind, const std::vector<int> &rptr, int N, const int *cptr,
                             int cnum, int bs)
{
    SENK_REQUIRE(cnum > 0 && cptr[0] == 0 && (long long)cptr[cnum] * bs == N, "colour pointer does not cover N rows");
    std::vector<int> colour(N);
    for (int k = 0; k < cnum; k++) {
        SENK_REQUIRE(cptr[k + 1] >= cptr[k], "colour pointer not monotone");
        for (int p = cptr[k] * bs; p < cptr[k + 1] * bs; p++) colour[p] = k;
    }
    for (int i = 0; i < N; i++) {
        const int cs = i - i % bs;
        for (int j = rptr[i]; j < rptr[i + 1]; j++) {
            const int c = cind[j];
            SENK_REQUIRE(c >= 0 && c < N, "column out of range");
            if (c >= i) break;
            SENK_REQUIRE(c >= cs || colour[c] < colour[i],
                         "row " + std::to_string(i) + " reads row " + std::to_string(c) +
                             " of its own colour: the matrix is not in the schedule's order");
        }
    }
    FactorSchedule f;
    f.rows.resize(N);
    for (int i = 0; i < N; i++) f.rows[i] = i;
    f.phase_chains.assign(cptr, cptr + cnum + 1);
    f.bs = bs;
    return f;
}

template <typename T>
int dev_ilu0(T *val, const int *cind, const int *rptr, int N, const int *cptr, int cnum, int bsize,
             cudaStream_t s)
{
    SENK_REQUIRE(val && cind && rptr && N > 0, "null argument or empty matrix");
    std::vector<int> hr(N + 1);
    SENK_CUDA(cudaMemcpyAsync(hr.data(), rptr, sizeof(int) * (N + 1), cudaMemcpyDeviceToHost, s));
    SENK_CUDA(cudaStreamSynchronize(s));
    SENK_REQUIRE(hr[0] == 0, "rptr must start at 0");
    for (int i = 0; i < N; i++) SENK_REQUIRE(hr[i + 1] >= hr[i], "rptr not monotone");
    std::vector<int> hc(hr[N]);
    SENK_CUDA(cudaMemcpyAsync(hc.data(), cind, sizeof(int) * hc.size(), cudaMemcpyDeviceToHost, s));
    SENK_CUDA(cudaStreamSynchronize(s));
    for (int i = 0; i < N; i++)
        for (int j = hr[i]; j + 1 < hr[i + 1]; j++) SENK_REQUIRE(hc[j] < hc[j + 1], "columns must be sorted");
    const FactorSchedule f = cptr ? colour_chains(hc, hr, N, cptr, cnum, bsize) : level_sets(hc, hr, N);
    DevBuf<int> rows(N), status(1);
    rows.upload(f.rows.data(), N, s);
    SENK_CUDA(cudaMemsetAsync(status.p, 0, sizeof(int), s));
    for (size_t p = 0; p + 1 < f.phase_chains.size(); p++) {
        const int c0 = f.phase_chains[p], nch = f.phase_chains[p + 1] - c0;
        if (nch <= 0) continue;
        k_ilu0_chains<T><<<ceil_div(nch, 128), 128, 0, s>>>(val, cind, rptr, rows.p, c0, nch, f.bs, status.p);
        SENK_LAUNCH_CHECK();
    }
    int h = 0;
    SENK_CUDA(cudaMemcpyAsync(&h, status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    SENK_CUDA(cudaStreamSynchronize(s));
    if (h) {
        set_last_error("senk_dev_ilu0: Error: Ilu0, 0 pivot");
        return kErrZeroPivot;
    }
    return kOk;
}

}  // namespace

}  // namespace senkgpu

using namespace senkgpu;

extern "C" {

int senk_dev_ilu0_d(double *val, const int *cind, const int *rptr, int N, const int *cptr, int cnum, int bsize,
                    void *stream)
{
    return guarded("senk_dev_ilu0_d", [&] {
        return dev_ilu0<double>(val, cind, rptr, N, cptr, cnum, bsize, (cudaStream_t)stream);
    });
}

int senk_dev_ilu0_s(float *val, const int *cind, const int *rptr, int N, const int *cptr, int cnum, int bsize,
                    void *stream)
{
    return guarded("senk_dev_ilu0_s", [&] {
        return dev_ilu0<float>(val, cind, rptr, N, cptr, cnum, bsize, (cudaStream_t)stream);
    });
}

}  // extern "C"
