// Compact chain layout of a triangular factor for the dataflow sweeps
// (k_sweep_wf in kernels.cuh). Host-only code: it builds plain arrays that the
// plan uploads, and a CPU emulation of the kernel can build them too.
//
// The schedule is a list of colours (position ranges, in processing order); a
// chain is `bs` consecutive rows of one colour, solved in order. The chains of
// each colour are sorted by their entry counts (external first, then in-chain,
// both descending) and taken 32 at a time into groups, lane q = chain q. Group
// block at `off`: external entry k of lane q at off + k*32 + q for
// k < E_q <= emax (slot-major, so a warp taking one entry of every chain
// reads 32 consecutive words); then the in-chain entries chain after chain,
// entry k of lane q at off + emax*32 + ibase_q + k with ibase_q the sum of
// I over the lanes before q (a chain's rows, handled by consecutive lanes,
// read consecutive words). Both parts list rows in solve order (ascending for L,
// descending for U) and each row's entries in the reference's subtraction
// order (include/senk_sparse.hpp:132-167: ascending columns for L, descending
// for U, the U diagonal kept apart as dinv). Column words: external
// (row << 27) | column; in-chain (row << 8) | chain-local column. Per chain
// also 2*bs bytes: the external then the in-chain entry count of each
// chain-local row (rows in their natural order), for kernels that split a
// chain's rows over warps.
//
// chain_major: the external part instead chain after chain, entry k of lane q
// at off + q*emax + k, with emax rounded up to an odd number (the chains'
// streams then start in different shared-memory banks), for kernels whose
// lanes are the rows of one chain (k_sweep_rl); the chain descriptors then
// hold ibase_q in place of I ({first row, E | ibase_q << 16}), so that a lane
// finds its chain's in-chain entries from its own descriptor.
#pragma once

#include <vector_functions.h>
#include <vector_types.h>

#include <algorithm>
#include <climits>
#include <cstddef>
#include <stdexcept>
#include <string>
#include <vector>

namespace senkgpu {

struct WfGroup {
    int off;      // element offset of the group's block
    int emax;     // external slots (the widest chain's E)
    int imax;     // in-chain slots (the widest chain's I)
    int nchains;  // chains in this group (<= 32)
};
static_assert(sizeof(WfGroup) == 16, "WfGroup is one 16-byte load");

constexpr int kColBits = 27;  // external column words: (row << 27) | column
constexpr int kColMask = (1 << kColBits) - 1;

struct WfColour {
    int p0, p1;  // rows [p0, p1) of one colour
};

// Shared memory of one warp of k_sweep_wf for a block of `slots` slots
// (equals wf_warp_bytes in kernels.cuh with XT = VT).
template <typename VT>
size_t wf_bytes_for(int slots, int bs, bool upper)
{
    return ((size_t)slots * 32 * (4 + sizeof(VT)) + (size_t)bs * 32 * sizeof(VT) * (upper ? 2 : 1) + 8 + 15) / 16 *
           16;
}

template <typename VT>
struct WfLayout {
    std::vector<WfGroup> groups;  // in processing order
    std::vector<int2> chains;     // per group 32 x {first row, E | I << 16} (unused lanes {0, 0})
    std::vector<unsigned char> counts;  // per group 32 x 2*bs row counts (external, in-chain)
    std::vector<VT> val;          // block values
    std::vector<int> col;         // block column words
    std::vector<VT> dinv;         // U: inverted diagonal per row
    std::vector<VT> cdinv;        // U: the same per chain, chain after chain (32 x bs per group)
    std::vector<int> dep_ptr, dep_idx;  // groups each group reads from (all earlier)
    std::vector<int> colour_groups;     // group range of each colour (size colours + 1)
    std::vector<int> colour_slots;      // widest block of each colour
    int slots_max = 0;
    long long stored = 0;         // off-diagonal entries stored
};

// Builds the layout of one factor. colour_of[row]: the colour's index in
// processing order. Throws std::invalid_argument when the factor does not fit
// the schedule; returns false when a group's block would need more than
// `max_smem` bytes of shared memory per warp.
template <typename VT>
bool make_wf_layout(WfLayout<VT> &out, bool upper, int N, const VT *val, const int *cind, const int *rptr,
                    const std::vector<WfColour> &colours, int bs, const int *colour_of, size_t max_smem,
                    const int *rowmap = nullptr, bool chain_major = false)
{
    if (N > kColMask) throw std::invalid_argument("N too large for the compact sweep layout (2^27 rows)");
    if (bs < 1 || bs > 32 || N % bs) throw std::invalid_argument("chain length must divide N and be at most 32");
    if (rowmap && bs != 1) throw std::invalid_argument("a row map takes chains of one row");
    const int nb = N / bs;  // chains; chain b holds rows [b*bs, b*bs + bs), or row rowmap[b]
    auto first_row = [&](int b) { return rowmap ? rowmap[b] : b * bs; };
    std::vector<int> E(nb), I(nb);
    int bad = -1;
#pragma omp parallel for schedule(static)
    for (int b = 0; b < nb; b++) {
        int ne = 0, ni = 0;
        bool ok = true;
        const int cs = first_row(b), ce = cs + bs;
        if (cs < 0 || cs >= N) ok = false;
        for (int row = cs; row < ce && ok; row++) {
            int j0 = rptr[row];
            const int j1 = rptr[row + 1];
            if (upper) {
                ok = j1 > j0 && cind[j0] == row;  // a U row starts with its diagonal
                j0++;
            }
            for (int j = j0; j < j1 && ok; j++) {
                const int c = cind[j];
                if (c < 0 || c >= N || (upper ? c <= row : c >= row)) ok = false;
                else if (c >= cs && c < ce) ni++;
                else if (colour_of[c] >= colour_of[row]) ok = false;  // must be final before this colour
                else ne++;
            }
        }
        for (int row = cs; row < ce && ok; row++) {  // at most 255 entries of each kind per row
            int re = 0, ri = 0;
            for (int j = rptr[row] + (upper ? 1 : 0); j < rptr[row + 1]; j++) {
                if (cind[j] >= cs && cind[j] < ce) ri++;
                else re++;
            }
            ok = re <= 255 && ri <= 255;
        }
        if (!ok || ne > 0xffff || ni > 0x7fff) {
#pragma omp atomic write
            bad = b;
        }
        E[b] = ne;
        I[b] = ni;
    }
    if (bad >= 0)
        throw std::invalid_argument(std::string(upper ? "U" : "L") + " factor rows of chain " + std::to_string(bad) +
                                    " do not fit the schedule (diagonal first in U, strictly triangular, columns "
                                    "of other chains in earlier colours)");
    // chains of each colour sorted by their counts, 32 to a group
    std::vector<WfGroup> gd;
    std::vector<int2> chv;
    std::vector<int> cg(1, 0);
    long long covered = 0;
    for (const WfColour &c : colours) {
        if (c.p0 % bs || c.p1 % bs || c.p1 < c.p0 || c.p0 < 0 || c.p1 > N)
            throw std::invalid_argument("colour range not made of whole chains");
        covered += c.p1 - c.p0;
        std::vector<int> ch;
        for (int b = c.p0 / bs; b < c.p1 / bs; b++) ch.push_back(b);
        std::stable_sort(ch.begin(), ch.end(),
                         [&](int a, int b) { return E[a] != E[b] ? E[a] > E[b] : I[a] > I[b]; });
        for (size_t q0 = 0; q0 < ch.size(); q0 += 32) {
            WfGroup d{};
            d.nchains = (int)std::min<size_t>(32, ch.size() - q0);
            for (int q = 0; q < 32; q++) {
                if (q < d.nchains) {
                    const int b = ch[q0 + q];
                    d.emax = std::max(d.emax, E[b]);
                    d.imax = std::max(d.imax, I[b]);
                    chv.push_back(make_int2(first_row(b), E[b] | (I[b] << 16)));
                } else {
                    chv.push_back(make_int2(0, 0));
                }
            }
            gd.push_back(d);
        }
        cg.push_back((int)gd.size());
    }
    if (covered != N) throw std::invalid_argument("colours do not cover the N rows");
    const int ng = (int)gd.size();
    int smax = 0;
    long long off = 0;
    for (WfGroup &d : gd) {
        if (chain_major && d.emax > 0) d.emax |= 1;
        d.off = (int)off;
        off += (long long)(d.emax + d.imax) * 32;
        if (off >= INT_MAX) throw std::invalid_argument("factor too large for 32-bit slot offsets");
        smax = std::max(smax, d.emax + d.imax);
    }
    if (wf_bytes_for<VT>(smax, bs, upper) > max_smem) return false;
    out.val.assign((size_t)off, VT(0));
    out.col.assign((size_t)off, 0);
    out.counts.assign((size_t)ng * 32 * 2 * bs, 0);
    out.cdinv.assign(upper ? (size_t)ng * 32 * bs : 0, VT(0));
    out.dinv.assign(upper ? N : 0, VT(0));
    std::vector<int> owner(N, -1);  // group of each row
    long long stored = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : stored)
    for (int g = 0; g < ng; g++) {
        const WfGroup d = gd[g];
        for (int q = 0; q < d.nchains; q++) {
            const int r0 = chv[(size_t)g * 32 + q].x;
            int ke = 0, ki = 0;
            int ibase = 0;
            for (int q2 = 0; q2 < q; q2++) ibase += (int)((unsigned)chv[(size_t)g * 32 + q2].y >> 16);
            for (int st = 0; st < bs; st++) {
                const int l = upper ? bs - 1 - st : st;  // rows in solve order
                const int row = r0 + l;
                owner[row] = g;
                unsigned char *cnt = out.counts.data() + ((size_t)g * 32 + q) * 2 * bs;
                auto put = [&](int j) {
                    const int c = cind[j];
                    if (c >= r0 && c < r0 + bs) {
                        cnt[bs + l]++;
                        const long long at = d.off + (long long)d.emax * 32 + ibase + ki++;
                        out.col[at] = (l << 8) | (c - r0);
                        out.val[at] = val[j];
                    } else {
                        cnt[l]++;
                        const long long at = chain_major ? d.off + (long long)q * d.emax + ke++
                                                         : d.off + (long long)(ke++) * 32 + q;
                        out.col[at] = (int)(((unsigned)l << kColBits) | (unsigned)c);
                        out.val[at] = val[j];
                    }
                    stored++;
                };
                if (upper) {
                    out.dinv[row] = val[rptr[row]];
                    out.cdinv[((size_t)g * 32 + q) * bs + l] = val[rptr[row]];
                    for (int j = rptr[row + 1] - 1; j >= rptr[row] + 1; j--) put(j);
                } else {
                    for (int j = rptr[row]; j < rptr[row + 1]; j++) put(j);
                }
            }
        }
    }
    // dependencies: the groups owning each group's external columns (all earlier)
    std::vector<std::vector<int>> deps(ng);
    bad = -1;
#pragma omp parallel
    {
        std::vector<int> seen(ng, -1);
#pragma omp for schedule(dynamic, 16)
        for (int g = 0; g < ng; g++) {
            for (int q = 0; q < gd[g].nchains; q++) {
                const int r0 = chv[(size_t)g * 32 + q].x;
                for (int row = r0; row < r0 + bs; row++) {
                    for (int j = rptr[row] + (upper ? 1 : 0); j < rptr[row + 1]; j++) {
                        const int c = cind[j];
                        if (c >= r0 && c < r0 + bs) continue;
                        const int o = owner[c];
                        if (o < 0 || o >= g) {
#pragma omp atomic write
                            bad = g;
                            continue;
                        }
                        if (seen[o] != g) {
                            seen[o] = g;
                            deps[g].push_back(o);
                        }
                    }
                }
            }
        }
    }
    if (bad >= 0)
        throw std::invalid_argument("group " + std::to_string(bad) + " reads a group that is not solved before it");
    out.dep_ptr.assign(ng + 1, 0);
    for (int g = 0; g < ng; g++) out.dep_ptr[g + 1] = out.dep_ptr[g] + (int)deps[g].size();
    out.dep_idx.clear();
    out.dep_idx.reserve(out.dep_ptr[ng]);
    for (int g = 0; g < ng; g++) out.dep_idx.insert(out.dep_idx.end(), deps[g].begin(), deps[g].end());
    out.colour_slots.assign(cg.size() - 1, 0);
    for (size_t c = 0; c + 1 < cg.size(); c++)
        for (int g = cg[c]; g < cg[c + 1]; g++)
            out.colour_slots[c] = std::max(out.colour_slots[c], gd[g].emax + gd[g].imax);
    if (chain_major)
        for (int g = 0; g < ng; g++) {
            unsigned ibase = 0;
            for (int q = 0; q < 32; q++) {
                int2 &c = chv[(size_t)g * 32 + q];
                const unsigned I = (unsigned)c.y >> 16;
                c.y = (int)(((unsigned)c.y & 0xffffu) | (ibase << 16));
                ibase += I;
            }
        }
    out.colour_groups = std::move(cg);
    out.groups = std::move(gd);
    out.chains = std::move(chv);
    out.slots_max = smax;
    out.stored = stored;
    return true;
}

}  // namespace senkgpu
