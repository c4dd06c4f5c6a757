// ILUB: triangular sweeps on BCSR factors (include/senk_sparse.hpp:392-465
// sequential, 481-581 ABMC).
//
// Semantics kept from the reference, block row by block row (i = first row):
//  L: y[i..i+bnl) = x; for every block in ascending order and every column l of
//     it, all rows of the block row subtract bval * y[col]. The reference's row
//     loop is `omp simd`, built by g++ -O3 from vectors of two doubles: y[col]
//     is read again for each pair of rows (r, r+1), after the pairs before it
//     were updated. That is visible when a block holds a value on the diagonal:
//     Csr2Bcsr (include/senk_matrix.hpp:144-211) gives an empty L row the first
//     entry of the next row, so the first row of every block row without lower
//     entries carries one. Rows in a later pair than row `col` see its updated
//     value, rows in its own or an earlier pair the value before the step.
//  U: y[i..i+bnl) = x; the blocks right of the diagonal square in descending
//     order (their columns ascending within a block) as above; then the
//     bnl/bnw diagonal blocks column by column from the right: y[idx] *=
//     (inverted diagonal), then every row above subtracts bval * y[idx].
// One group of G lanes (G = bnl rounded up to a power of two) sweeps one chain;
// lane k holds row i+k. A column inside the block row is read from its lane by
// a shuffle before the step's update; any other column is final in global
// memory (an earlier phase, or an earlier block row of the same chain, written
// by this group before its __syncwarp).
#include <algorithm>
#include <vector>

#include "device.hpp"

namespace senkgpu {

namespace {

template <int BNL>
constexpr int group_lanes()
{
    return BNL <= 1 ? 1 : BNL <= 2 ? 2 : BNL <= 4 ? 4 : BNL <= 8 ? 8 : BNL <= 16 ? 16 : 32;
}

template <typename T, int BNL, int BNW, bool UPPER>
__global__ void __launch_bounds__(kThreads)
k_ilub_sweep(const T *__restrict__ bval, const int *__restrict__ bcind, const int *__restrict__ brptr,
             const int2 *__restrict__ chains, int nch, const T *x, T *y, const int *gate)
{
    if (gated(gate)) return;
    constexpr int G = group_lanes<BNL>();
    constexpr int BS = BNL * BNW;
    constexpr int BREM = BNL / BNW;
    const int lane = threadIdx.x % G;
    const int gid = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) / G);
    if (gid >= nch) return;  // uniform over the group
    const unsigned mask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (((threadIdx.x & 31) / G) * G));
    const int2 ch = chains[gid];
    for (int q = 0; q < ch.y; q++) {
        const int br = UPPER ? ch.x + ch.y - 1 - q : ch.x + q;
        const int i = br * BNL;
        T t = lane < BNL ? x[i + lane] : T(0);
        const int b0 = brptr[br], b1 = brptr[br + 1];
        // Blocks are taken kBatch at a time: their columns, values and (for
        // columns outside this block row) y entries are all loaded before the
        // first subtraction, which then run in the blocks' order as before.
        constexpr int kBatch = 4;
        if (!UPPER) {
            for (int j0 = b0; j0 < b1; j0 += kBatch) {
                int xb[kBatch];
                T vv[kBatch][BNW], yy[kBatch][BNW];
#pragma unroll
                for (int u = 0; u < kBatch; u++) xb[u] = j0 + u < b1 ? bcind[j0 + u] * BNW : i;
#pragma unroll
                for (int u = 0; u < kBatch; u++)
#pragma unroll
                    for (int l = 0; l < BNW; l++) {
                        const int rel = xb[u] + l - i;
                        const bool live = j0 + u < b1;
                        vv[u][l] = live && lane < BNL ? bval[(size_t)(j0 + u) * BS + l * BNL + lane] : T(0);
                        yy[u][l] = live && !(rel >= 0 && rel < BNL) ? y[xb[u] + l] : T(0);
                    }
#pragma unroll
                for (int u = 0; u < kBatch; u++) {
                    if (j0 + u >= b1) break;
#pragma unroll
                    for (int l = 0; l < BNW; l++) {
                        const int rel = xb[u] + l - i;
                        const T v = vv[u][l];
                        if (rel >= 0 && rel < BNL) {
                            const T s0 = __shfl_sync(mask, t, rel, G);
                            const T t0 = t - v * s0;
                            const T s1 = __shfl_sync(mask, t0, rel, G);  // y[col] after its own pair
                            t = (lane >> 1) > (rel >> 1) ? t - v * s1 : t0;
                        } else {
                            t -= v * yy[u][l];
                        }
                    }
                }
            }
        } else {
            // blocks right of the diagonal square, from the last one down
            for (int j0 = b1 - 1; j0 >= b0 + BREM; j0 -= kBatch) {
                T vv[kBatch][BNW], yy[kBatch][BNW];
#pragma unroll
                for (int u = 0; u < kBatch; u++) {
                    const int j = j0 - u;
                    const bool live = j >= b0 + BREM;
                    const int xb = live ? bcind[j] * BNW : 0;
#pragma unroll
                    for (int l = 0; l < BNW; l++) {
                        vv[u][l] = live && lane < BNL ? bval[(size_t)j * BS + l * BNL + lane] : T(0);
                        yy[u][l] = live ? y[xb + l] : T(0);
                    }
                }
#pragma unroll
                for (int u = 0; u < kBatch; u++) {
                    if (j0 - u < b0 + BREM) break;
#pragma unroll
                    for (int l = 0; l < BNW; l++) t -= vv[u][l] * yy[u][l];
                }
            }
#pragma unroll
            for (int m = BREM - 1; m >= 0; m--) {
                const T *blk = bval + (size_t)(b0 + m) * BS;
#pragma unroll
                for (int jj = BNW - 1; jj >= 0; jj--) {
                    const int idx = m * BNW + jj;
                    if (lane == idx) t *= blk[jj * BNL + idx];
                    const T s = __shfl_sync(mask, t, idx, G);
                    if (lane < idx) t -= blk[jj * BNL + lane] * s;
                }
            }
        }
        if (lane < BNL) y[i + lane] = t;
        __syncwarp(mask);
    }
}

#define SENK_ILUB_SHAPES(X) X(1, 1) X(2, 1) X(2, 2) X(3, 3) X(4, 1) X(4, 2) X(4, 4) X(8, 1) X(8, 2)

bool shape_supported(int bnl, int bnw)
{
#define X(R, C) if (bnl == R && bnw == C) return true;
    SENK_ILUB_SHAPES(X)
#undef X
    return false;
}

int lanes_of(int bnl) { return bnl <= 1 ? 1 : bnl <= 2 ? 2 : bnl <= 4 ? 4 : bnl <= 8 ? 8 : bnl <= 16 ? 16 : 32; }

// Checks one factor against the schedule: every column a block row reads from
// outside itself must be final when the block row runs (an earlier phase, or
// an earlier block row of its own chain). The reference would race otherwise.
void check_factor(bool upper, int nbr, int bnl, int bnw, const int *bcind, const int *brptr,
                  const std::vector<int2> &chains, const std::vector<int> &phase_chains, const char *name)
{
    const int nbc = nbr * bnl / bnw, brem = bnl / bnw;
    SENK_REQUIRE(brptr[0] == 0, std::string(name) + ": brptr[0] must be 0");
    for (int br = 0; br < nbr; br++) {
        SENK_REQUIRE(brptr[br + 1] >= brptr[br], std::string(name) + ": brptr not monotonic");
        for (int j = brptr[br]; j < brptr[br + 1]; j++)
            SENK_REQUIRE(bcind[j] >= 0 && bcind[j] < nbc, std::string(name) + ": block column out of range");
        if (upper) {
            SENK_REQUIRE(brptr[br + 1] - brptr[br] >= brem,
                         std::string(name) + ": block row without its diagonal square");
            for (int m = 0; m < brem; m++)
                SENK_REQUIRE(bcind[brptr[br] + m] == br * brem + m,
                             std::string(name) + ": the leading blocks of a row must be its diagonal square");
        }
    }
    // done[br]: 2 = finished in an earlier phase; 1 = finished earlier in the
    // chain being checked
    std::vector<unsigned char> done(nbr, 0);
    const int P = (int)phase_chains.size() - 1;
    for (int pi = 0; pi < P; pi++) {
        const int p = upper ? P - 1 - pi : pi;
        for (int c = phase_chains[p]; c < phase_chains[p + 1]; c++) {
            const int2 ch = chains[c];
            for (int q = 0; q < ch.y; q++) {
                const int br = upper ? ch.x + ch.y - 1 - q : ch.x + q;
                const int j0 = brptr[br] + (upper ? brem : 0);
                for (int j = j0; j < brptr[br + 1]; j++) {
                    for (int l = 0; l < bnw; l++) {
                        const int col = bcind[j] * bnw + l, cbr = col / bnl;
                        if (cbr == br) {
                            SENK_REQUIRE(!upper, std::string(name) + ": U block right of the diagonal square "
                                                                     "reaches into its own block row");
                            continue;
                        }
                        SENK_REQUIRE(done[cbr] != 0, std::string(name) + ": block row " + std::to_string(br) +
                                                         " reads row " + std::to_string(col) +
                                                         " before the schedule has finished it");
                    }
                }
                done[br] = 1;
            }
            // rows of this chain may not be read by the other chains of the phase
            for (int q = 0; q < ch.y; q++) done[ch.x + q] = 0;
        }
        for (int c = phase_chains[p]; c < phase_chains[p + 1]; c++)
            for (int q = 0; q < chains[c].y; q++) done[chains[c].x + q] = 2;
    }
    for (int br = 0; br < nbr; br++) SENK_REQUIRE(done[br] == 2, std::string(name) + ": block row not scheduled");
}

}  // namespace

template <typename T>
void IlubPlan<T>::build(int N, int bnl_, int bnw_, const T *blval, const int *blcind, const int *blrptr,
                        const T *buval, const int *bucind, const int *burptr, const int *cptr, int cnum, int bsize,
                        cudaStream_t s)
{
    SENK_REQUIRE(shape_supported(bnl_, bnw_), "ILUB block shape " + std::to_string(bnl_) + "x" +
                                                  std::to_string(bnw_) +
                                                  " is not built (1x1 2x1 2x2 3x3 4x1 4x2 4x4 8x1 8x2)");
    SENK_REQUIRE(N > 0 && N % bnl_ == 0, "N must be a multiple of bnl");
    SENK_REQUIRE(blval && blcind && blrptr && buval && bucind && burptr, "null BCSR factor array");
    n = N;
    bnl = bnl_;
    bnw = bnw_;
    nbr = N / bnl;
    std::vector<int2> ch;
    phase_chains.assign(1, 0);
    if (cptr) {
        SENK_REQUIRE(cnum > 0 && bsize > 0 && bsize % bnl == 0, "ABMC bsize must be a positive multiple of bnl");
        SENK_REQUIRE(cptr[0] == 0, "cptr[0] must be 0");
        const int per = bsize / bnl;
        for (int c = 0; c < cnum; c++) {
            SENK_REQUIRE(cptr[c + 1] >= cptr[c], "cptr not monotonic");
            for (int blk = cptr[c]; blk < cptr[c + 1]; blk++) {
                const long long first = (long long)blk * per;
                SENK_REQUIRE(first < nbr, "colour block beyond N");
                ch.push_back(make_int2((int)first, (int)std::min<long long>(per, nbr - first)));
            }
            phase_chains.push_back((int)ch.size());
        }
    } else {
        ch.push_back(make_int2(0, nbr));
        phase_chains.push_back(1);
    }
    check_factor(false, nbr, bnl, bnw, blcind, blrptr, ch, phase_chains, "ILUB L factor");
    check_factor(true, nbr, bnl, bnw, bucind, burptr, ch, phase_chains, "ILUB U factor");
    lblocks = blrptr[nbr];
    ublocks = burptr[nbr];
    const size_t bs = (size_t)bnl * bnw;
    auto put = [s](auto &buf, const auto *h, size_t count) {
        buf.alloc(count);
        buf.upload(h, count, s);
    };
    put(lval, blval, (size_t)lblocks * bs);
    put(lcind, blcind, (size_t)lblocks);
    put(lrptr, blrptr, (size_t)nbr + 1);
    put(uval, buval, (size_t)ublocks * bs);
    put(ucind, bucind, (size_t)ublocks);
    put(urptr, burptr, (size_t)nbr + 1);
    put(chains, ch.data(), ch.size());
    SENK_CUDA(cudaStreamSynchronize(s));  // the host vectors go out of scope
}

template <typename T>
void IlubPlan<T>::sweep(bool upper, const T *x, T *y, cudaStream_t s, const int *gate) const
{
    const int P = (int)phase_chains.size() - 1;
    const int G = lanes_of(bnl);
    for (int pi = 0; pi < P; pi++) {
        const int p = upper ? P - 1 - pi : pi;
        const int c0 = phase_chains[p], nch = phase_chains[p + 1] - c0;
        if (nch == 0) continue;
        const long long lanes = (long long)nch * G;
        const int threads = (int)std::min<long long>(kThreads, (lanes + 31) / 32 * 32);
        const int grid = ceil_div(lanes, threads);
#define X(R, C)                                                                                               \
    if (bnl == R && bnw == C) {                                                                               \
        if (upper)                                                                                            \
            k_ilub_sweep<T, R, C, true><<<grid, threads, 0, s>>>(uval.p, ucind.p, urptr.p, chains.p + c0, nch, x, \
                                                                 y, gate);                                    \
        else                                                                                                  \
            k_ilub_sweep<T, R, C, false><<<grid, threads, 0, s>>>(lval.p, lcind.p, lrptr.p, chains.p + c0, nch, \
                                                                  x, y, gate);                                \
    } else
        SENK_ILUB_SHAPES(X)
#undef X
        throw ArgError("unsupported ILUB block shape");
        SENK_LAUNCH_CHECK();
    }
}

template <typename T>
long long IlubPlan<T>::apply_bytes() const
{
    const long long vb = sizeof(T), bs = (long long)bnl * bnw;
    // blocks (values + block column) and block row pointers of both factors;
    // x read, y written by L, read and written by U
    return (lblocks + ublocks) * (bs * vb + 4) + 2LL * (nbr + 1) * 4 + 4LL * n * vb;
}

template struct IlubPlan<double>;
template struct IlubPlan<float>;

void learned_apply(void *net, const void *sys, const double *v, double *out, cudaStream_t s);

template <typename T>
void System<T>::precondition(const T *v, T *out, const int *gate)
{
    precondition_base(v, out, gate);
    if constexpr (std::is_same<T, double>::value) {
        if (learned) learned_apply(learned, this, v, out, stream);
    }
}

template <typename T>
void System<T>::precondition_base(const T *v, T *out, const int *gate)
{
    if (pcb) pcb->apply(v, out, stream, gate);
    else if (pc) pc->apply(v, out, stream, gate);
    else
        k_elementwise<T, 4><<<stream_grid(n, kThreads, 8), kThreads, 0, stream>>>(T(0), nullptr, 1.0, T(0), v, out,
                                                                                  nullptr, n, gate);
    SENK_LAUNCH_CHECK();
}

template <typename T>
void System<T>::check_pc() const
{
    if (pc) pc->check_status(stream);
}

template void System<double>::precondition(const double *, double *, const int *);
template void System<float>::precondition(const float *, float *, const int *);
template void System<double>::precondition_base(const double *, double *, const int *);
template void System<float>::precondition_base(const float *, float *, const int *);
template void System<double>::check_pc() const;
template void System<float>::check_pc() const;

}  // namespace senkgpu
