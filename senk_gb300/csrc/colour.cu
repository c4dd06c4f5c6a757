// ABMC and AMC orderings on the device: the reference's GetABMCPermutation
// with simple blocking and GetAMCPermutation (include/senk_graph.hpp:250-334,
// isSym = false), computed in parallel with the same result, and the device
// form of Reordering (include/senk_matrix.hpp:703-730).
//
// The reference blocks the rows (here: bsize consecutive rows, its "simple"
// blocking; AMC is bsize 1), builds the symmetric block adjacency (pattern
// plus transpose) and colours it greedily: colour 1 takes, in index order,
// every block not adjacent to a block already taken for colour 1; colour 2
// does the same among the rest, and so on (Coloring, senk_graph.hpp:218-238).
// Each colour is therefore the lexicographically first maximal independent
// set of the uncoloured blocks. Rounds compute that set in parallel: a
// candidate block joins when none of its candidate neighbours has a smaller
// number, and the neighbours of the blocks that joined stop being candidates.
// A block joins exactly when all its smaller neighbours have been excluded,
// which is the greedy sweep's rule, so the colours are the reference's. The
// rounds follow the chains of smaller neighbours: about the graph's diameter
// in the index order (a few hundred for a 3D grid), issued in batches between
// host checks. The ordering step is the reference's: colours in order, blocks
// of a colour in ascending number, the rows of a block in order (LP: new ->
// old, RP: old -> new, size_color in blocks).
#include <algorithm>
#include <vector>

#include "device.hpp"

namespace senkgpu {

namespace {

constexpr int kMaxBlockDegree = 128;  // distinct neighbour blocks of one block
constexpr int kMaxColours = 255;
constexpr int kRoundBatch = 16;  // independent-set rounds between checks on the host

// Exclusive scan of n ints (out may alias in), in three launches: per-CTA
// sums, a one-CTA scan of those sums, then the per-CTA scans with their
// offsets. Returns nothing; total = out[n-1] + in[n-1] is left to the caller.
constexpr int kScanItems = 1024;  // per CTA of 256 threads, 4 each

__global__ void __launch_bounds__(256) k_scan_sums(const int *__restrict__ in, int n, int *__restrict__ sums)
{
    __shared__ int sh[8];
    const int base = blockIdx.x * kScanItems;
    int s = 0;
    for (int k = threadIdx.x; k < kScanItems; k += 256)
        if (base + k < n) s += in[base + k];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < 8; w++) t += sh[w];
        sums[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(256) k_scan_offsets(int *sums, int nb)
{
    // one CTA: exclusive scan of nb sums, in chunks of 256
    __shared__ int sh[256];
    int carry = 0;
    for (int b0 = 0; b0 < nb; b0 += 256) {
        const int i = b0 + threadIdx.x;
        const int v = i < nb ? sums[i] : 0;
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < 256; o <<= 1) {
            const int t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
            __syncthreads();
            sh[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < nb) sums[i] = carry + sh[threadIdx.x] - v;
        const int total = sh[255];
        __syncthreads();
        carry += total;
    }
}

__global__ void __launch_bounds__(256)
k_scan_apply(const int *__restrict__ in, int n, const int *__restrict__ offs, int *__restrict__ out)
{
    // each thread scans 4 consecutive items; the threads' sums are scanned in shared memory
    __shared__ int sh[256];
    const int base = blockIdx.x * kScanItems + threadIdx.x * 4;
    int v[4], s = 0;
#pragma unroll
    for (int u = 0; u < 4; u++) {
        v[u] = base + u < n ? in[base + u] : 0;
        s += v[u];
    }
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < 256; o <<= 1) {
        const int t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
        __syncthreads();
        sh[threadIdx.x] += t;
        __syncthreads();
    }
    int run = offs[blockIdx.x] + sh[threadIdx.x] - s;
#pragma unroll
    for (int u = 0; u < 4; u++) {
        if (base + u < n) out[base + u] = run;
        run += v[u];
    }
}

void exclusive_scan(const int *in, int *out, int n, DevBuf<int> &tmp, cudaStream_t s)
{
    const int nb = (n + kScanItems - 1) / kScanItems;
    if (tmp.n < (size_t)std::max(nb, 1)) tmp.alloc(std::max(nb, 1));
    k_scan_sums<<<nb, 256, 0, s>>>(in, n, tmp.p);
    k_scan_offsets<<<1, 256, 0, s>>>(tmp.p, nb);
    k_scan_apply<<<nb, 256, 0, s>>>(in, n, tmp.p, out);
    SENK_LAUNCH_CHECK();
}

// Distinct neighbour blocks of block b (rows [b*bs, (b+1)*bs)), itself
// excluded, sorted; one thread per block. count only (out == nullptr) or fill.
__global__ void __launch_bounds__(128)
k_block_pattern(const int *__restrict__ cind, const int *__restrict__ rptr, int nb, int bs, const int *__restrict__ off,
                int *__restrict__ out, int *__restrict__ deg, int *status)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    int nbr[kMaxBlockDegree];
    int k = 0;
    for (int r = b * bs; r < (b + 1) * bs; r++) {
        for (int j = rptr[r]; j < rptr[r + 1]; j++) {
            const int c = cind[j] / bs;
            if (c == b) continue;
            // insertion into the sorted list, skipping duplicates
            int q = k;
            while (q > 0 && nbr[q - 1] > c) q--;
            if (q > 0 && nbr[q - 1] == c) continue;
            if (k == kMaxBlockDegree) {
                atomicExch(status, 1);
                return;
            }
            for (int t = k; t > q; t--) nbr[t] = nbr[t - 1];
            nbr[q] = c;
            k++;
        }
    }
    if (out) {
        for (int t = 0; t < k; t++) out[off[b] + t] = nbr[t];
    } else {
        deg[b] = k;
    }
}

// Transpose of the block pattern: in-degree counts, then an unordered fill.
__global__ void __launch_bounds__(256)
k_pattern_indeg(const int *__restrict__ pcol, const int *__restrict__ prow, int nb, int *__restrict__ indeg)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    for (int j = prow[b]; j < prow[b + 1]; j++) atomicAdd(indeg + pcol[j], 1);
}

__global__ void __launch_bounds__(256)
k_pattern_transpose(const int *__restrict__ pcol, const int *__restrict__ prow, int nb, const int *__restrict__ toff,
                    int *__restrict__ tfill, int *__restrict__ tcol)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    for (int j = prow[b]; j < prow[b + 1]; j++) {
        const int c = pcol[j];
        tcol[toff[c] + atomicAdd(tfill + c, 1)] = b;
    }
}

// Symmetric adjacency row b = sorted union of pattern row b and transposed row
// b (whose order is unsorted: sorted here first). count or fill.
__global__ void __launch_bounds__(128)
k_adjacency(const int *__restrict__ pcol, const int *__restrict__ prow, int *__restrict__ tcol,
            const int *__restrict__ trow, int nb, const int *__restrict__ aoff, int *__restrict__ acol,
            int *__restrict__ adeg)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const int t0 = trow[b], t1 = trow[b + 1];
    if (!acol) {  // sort the transposed row in place (insertion; rows are short)
        for (int i = t0 + 1; i < t1; i++) {
            const int v = tcol[i];
            int q = i - 1;
            while (q >= t0 && tcol[q] > v) {
                tcol[q + 1] = tcol[q];
                q--;
            }
            tcol[q + 1] = v;
        }
    }
    int i = prow[b], j = t0, k = 0;
    const int ie = prow[b + 1];
    while (i < ie || j < t1) {
        int v;
        if (j >= t1 || (i < ie && pcol[i] < tcol[j])) v = pcol[i++];
        else if (i >= ie || tcol[j] < pcol[i]) v = tcol[j++];
        else {
            v = pcol[i++];
            j++;
        }
        if (acol) acol[aoff[b] + k] = v;
        k++;
    }
    if (!acol) adeg[b] = k;
}

// One round of colour c: candidates (cand = 1) without a smaller candidate
// neighbour take colour c.
__global__ void __launch_bounds__(256)
k_mis_select(const int *__restrict__ acol, const int *__restrict__ aoff, int nb, const unsigned char *__restrict__ cand,
             int *__restrict__ colour, int c)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb || !cand[b]) return;
    // rows of the adjacency are sorted: only the neighbours below b matter
    for (int j = aoff[b]; j < aoff[b + 1]; j++) {
        const int o = acol[j];
        if (o >= b) break;
        if (cand[o]) return;
    }
    colour[b] = c;
}

// After a round: chosen blocks and their neighbours leave the candidates;
// *left counts the candidates that remain.
__global__ void __launch_bounds__(256)
k_mis_prune(const int *__restrict__ acol, const int *__restrict__ aoff, int nb, unsigned char *__restrict__ cand,
            const int *__restrict__ colour, int c, int *left)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb || !cand[b]) return;
    bool keep = colour[b] == 0;
    for (int j = aoff[b]; keep && j < aoff[b + 1]; j++) keep = colour[acol[j]] != c;
    if (!keep) cand[b] = 0;
    else atomicAdd(left, 1);
}

// Candidates of the next colour: the uncoloured blocks; *left counts them.
__global__ void __launch_bounds__(256)
k_mis_reset(int nb, unsigned char *__restrict__ cand, const int *__restrict__ colour, int *left)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const bool u = colour[b] == 0;
    cand[b] = u;
    if (u) atomicAdd(left, 1);
}

__global__ void __launch_bounds__(256)
k_colour_flag(const int *__restrict__ colour, int nb, int c, int *__restrict__ flag)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < nb) flag[b] = colour[b] == c;
}

// Blocks of colour c go to positions base + rank (rank = exclusive scan of the
// colour's flags); LP/RP for their rows.
__global__ void __launch_bounds__(256)
k_colour_place(const int *__restrict__ colour, const int *__restrict__ rank, int nb, int c, int base, int bs,
               int *__restrict__ LP, int *__restrict__ RP)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb || colour[b] != c) return;
    const int nbk = base + rank[b];
    for (int r = 0; r < bs; r++) {
        LP[nbk * bs + r] = b * bs + r;
        RP[b * bs + r] = nbk * bs + r;
    }
}

// Reordering: new row i holds old row LP[i] with columns RP[col], sorted.
__global__ void __launch_bounds__(256)
k_reorder_len(const int *__restrict__ rptr, const int *__restrict__ LP, int n, int *__restrict__ len)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) len[i] = rptr[LP[i] + 1] - rptr[LP[i]];
}

template <typename T>
__global__ void __launch_bounds__(128)
k_reorder_rows(const T *__restrict__ val, const int *__restrict__ cind, const int *__restrict__ rptr,
               const int *__restrict__ LP, const int *__restrict__ RP, int n, T *__restrict__ oval,
               int *__restrict__ ocind, const int *__restrict__ orptr)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int r = LP[i], s = rptr[r], len = rptr[r + 1] - s, o = orptr[i];
    for (int k = 0; k < len; k++) {
        const int c = RP[cind[s + k]];
        const T v = val[s + k];
        int q = k - 1;
        while (q >= 0 && ocind[o + q] > c) {
            ocind[o + q + 1] = ocind[o + q];
            oval[o + q + 1] = oval[o + q];
            q--;
        }
        ocind[o + q + 1] = c;
        oval[o + q + 1] = v;
    }
}

int grid_of(long long n, int threads) { return (int)std::max<long long>(1, (n + threads - 1) / threads); }

int get_int(const int *p, cudaStream_t s)
{
    int h = 0;
    SENK_CUDA(cudaMemcpyAsync(&h, p, sizeof(int), cudaMemcpyDeviceToHost, s));
    SENK_CUDA(cudaStreamSynchronize(s));
    return h;
}

// The device ABMC ordering; see the file comment. LP, RP: device arrays of N.
// Returns the colour count; size_color (host) gets num_color + 1 entries.
int dev_abmc(const int *cind, const int *rptr, int N, int bs, std::vector<int> &size_color, int *LP, int *RP,
             cudaStream_t s)
{
    SENK_REQUIRE(cind && rptr && LP && RP && N > 0, "null argument or empty matrix");
    SENK_REQUIRE(bs >= 1 && N % bs == 0, "N must be a multiple of bsize");
    const int nb = N / bs;
    DevBuf<int> deg(nb + 1), poff(nb + 1), status(1), tmp;
    SENK_CUDA(cudaMemsetAsync(status.p, 0, sizeof(int), s));
    SENK_CUDA(cudaMemsetAsync(deg.p + nb, 0, sizeof(int), s));
    k_block_pattern<<<grid_of(nb, 128), 128, 0, s>>>(cind, rptr, nb, bs, nullptr, nullptr, deg.p, status.p);
    SENK_LAUNCH_CHECK();
    SENK_REQUIRE(get_int(status.p, s) == 0, "a block has more than 128 neighbour blocks; use the host ordering");
    exclusive_scan(deg.p, poff.p, nb + 1, tmp, s);
    const int pnnz = get_int(poff.p + nb, s);
    DevBuf<int> pcol(std::max(pnnz, 1));
    k_block_pattern<<<grid_of(nb, 128), 128, 0, s>>>(cind, rptr, nb, bs, poff.p, pcol.p, nullptr, status.p);
    // symmetric adjacency: pattern + its transpose
    DevBuf<int> indeg(nb + 1), toff(nb + 1), tfill(nb), tcol(std::max(pnnz, 1));
    SENK_CUDA(cudaMemsetAsync(indeg.p, 0, sizeof(int) * (nb + 1), s));
    SENK_CUDA(cudaMemsetAsync(tfill.p, 0, sizeof(int) * nb, s));
    k_pattern_indeg<<<grid_of(nb, 256), 256, 0, s>>>(pcol.p, poff.p, nb, indeg.p);
    exclusive_scan(indeg.p, toff.p, nb + 1, tmp, s);
    k_pattern_transpose<<<grid_of(nb, 256), 256, 0, s>>>(pcol.p, poff.p, nb, toff.p, tfill.p, tcol.p);
    DevBuf<int> adeg(nb + 1), aoff(nb + 1);
    SENK_CUDA(cudaMemsetAsync(adeg.p + nb, 0, sizeof(int), s));
    k_adjacency<<<grid_of(nb, 128), 128, 0, s>>>(pcol.p, poff.p, tcol.p, toff.p, nb, nullptr, nullptr, adeg.p);
    exclusive_scan(adeg.p, aoff.p, nb + 1, tmp, s);
    const int annz = get_int(aoff.p + nb, s);
    DevBuf<int> acol(std::max(annz, 1));
    k_adjacency<<<grid_of(nb, 128), 128, 0, s>>>(pcol.p, poff.p, tcol.p, toff.p, nb, aoff.p, acol.p, nullptr);
    SENK_LAUNCH_CHECK();
    // colours: maximal independent sets of the uncoloured blocks, one after the other
    DevBuf<int> colour(nb), left(1);
    DevBuf<unsigned char> cand(nb);
    SENK_CUDA(cudaMemsetAsync(colour.p, 0, sizeof(int) * nb, s));
    int c = 0;
    for (;;) {
        SENK_CUDA(cudaMemsetAsync(left.p, 0, sizeof(int), s));
        k_mis_reset<<<grid_of(nb, 256), 256, 0, s>>>(nb, cand.p, colour.p, left.p);
        if (get_int(left.p, s) == 0) break;
        c++;
        SENK_REQUIRE(c <= kMaxColours, "more than 255 colours");
        // rounds in batches; once no candidate is left a round does nothing
        for (int round = 0;; round += kRoundBatch) {
            SENK_REQUIRE(round <= nb, "independent-set rounds do not converge");
            for (int r = 0; r < kRoundBatch; r++) {
                k_mis_select<<<grid_of(nb, 256), 256, 0, s>>>(acol.p, aoff.p, nb, cand.p, colour.p, c);
                SENK_CUDA(cudaMemsetAsync(left.p, 0, sizeof(int), s));
                k_mis_prune<<<grid_of(nb, 256), 256, 0, s>>>(acol.p, aoff.p, nb, cand.p, colour.p, c, left.p);
            }
            if (get_int(left.p, s) == 0) break;
        }
    }
    const int nc = c;
    // ordering: colours in order, blocks of a colour in ascending number
    size_color.assign(nc + 1, 0);
    DevBuf<int> flag(nb + 1), rank(nb + 1);
    SENK_CUDA(cudaMemsetAsync(flag.p + nb, 0, sizeof(int), s));
    for (int k = 1; k <= nc; k++) {
        k_colour_flag<<<grid_of(nb, 256), 256, 0, s>>>(colour.p, nb, k, flag.p);
        exclusive_scan(flag.p, rank.p, nb + 1, tmp, s);
        k_colour_place<<<grid_of(nb, 256), 256, 0, s>>>(colour.p, rank.p, nb, k, size_color[k - 1], bs, LP, RP);
        size_color[k] = size_color[k - 1] + get_int(rank.p + nb, s);
    }
    SENK_LAUNCH_CHECK();
    SENK_REQUIRE(size_color[nc] == nb, "colouring left blocks unplaced");
    return nc;
}

template <typename T>
int dev_reordering(const T *val, const int *cind, const int *rptr, const int *LP, const int *RP, int N, T *oval,
                   int *ocind, int *orptr, cudaStream_t s)
{
    SENK_REQUIRE(val && cind && rptr && LP && RP && oval && ocind && orptr && N > 0, "null argument or empty matrix");
    DevBuf<int> len(N + 1), tmp;
    SENK_CUDA(cudaMemsetAsync(len.p + N, 0, sizeof(int), s));
    k_reorder_len<<<grid_of(N, 256), 256, 0, s>>>(rptr, LP, N, len.p);
    exclusive_scan(len.p, orptr, N + 1, tmp, s);
    k_reorder_rows<T><<<grid_of(N, 128), 128, 0, s>>>(val, cind, rptr, LP, RP, N, oval, ocind, orptr);
    SENK_LAUNCH_CHECK();
    SENK_CUDA(cudaStreamSynchronize(s));  // the scan's scratch is released on return
    return (int)kOk;
}

}  // namespace

}  // namespace senkgpu

using namespace senkgpu;

extern "C" {

int senk_dev_abmc_ordering(const int *cind, const int *rptr, int N, int bsize, int *num_color, int **size_color,
                           int *LP, int *RP, void *stream)
{
    return guarded("senk_dev_abmc_ordering", [&] {
        SENK_REQUIRE(num_color && size_color, "null output");
        std::vector<int> sc;
        const int nc = dev_abmc(cind, rptr, N, bsize, sc, LP, RP, (cudaStream_t)stream);
        *size_color = static_cast<int *>(std::malloc(sizeof(int) * sc.size()));
        SENK_REQUIRE(*size_color, "host allocation failed");
        std::copy(sc.begin(), sc.end(), *size_color);
        *num_color = nc;
        return (int)kOk;
    });
}

int senk_dev_reordering_d(const double *val, const int *cind, const int *rptr, const int *LP, const int *RP, int N,
                          double *oval, int *ocind, int *orptr, void *stream)
{
    return guarded("senk_dev_reordering_d", [&] {
        return dev_reordering<double>(val, cind, rptr, LP, RP, N, oval, ocind, orptr, (cudaStream_t)stream);
    });
}

int senk_dev_reordering_s(const float *val, const int *cind, const int *rptr, const int *LP, const int *RP, int N,
                          float *oval, int *ocind, int *orptr, void *stream)
{
    return guarded("senk_dev_reordering_s", [&] {
        return dev_reordering<float>(val, cind, rptr, LP, RP, N, oval, ocind, orptr, (cudaStream_t)stream);
    });
}

}  // extern "C"
