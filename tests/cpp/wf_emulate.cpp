// CPU emulation of the dataflow ILU sweep (k_sweep_wf) on the compact chain
// layout that the plan builds (senk_gb300/csrc/wf_layout.hpp): every access the
// kernel makes is repeated here with its index checked against the buffer it
// reads, groups run in processing order, and each gathered row is checked to be
// finished and owned by a group on the reading group's dependency list. Test
// code only: it runs no GPU code.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <set>
#include <vector>

#include "wf_layout.hpp"

using namespace senkgpu;

namespace {

template <typename VT>
int emulate(int N, const VT *val, const int *cind, const int *rptr, int upper, const int *cptr, int cnum, int bs,
            const VT *x, VT *y, char *err, int errlen, const int *rowmap = nullptr)
{
    auto fail = [&](const std::string &m) {
        std::snprintf(err, errlen, "%s", m.c_str());
        return 1;
    };
    try {
        std::vector<WfColour> colours;
        std::vector<int> colour_of(N);
        if (rowmap) {  // level sets in processing order: cptr holds their position ranges
            for (int k = 0; k < cnum; k++) {
                colours.push_back({cptr[k], cptr[k + 1]});
                for (int p = cptr[k]; p < cptr[k + 1]; p++) colour_of[rowmap[p]] = k;
            }
        } else {
            for (int k = 0; k < cnum; k++) {
                const int c = upper ? cnum - 1 - k : k;
                colours.push_back({cptr[c] * bs, cptr[c + 1] * bs});
                for (int p = cptr[c] * bs; p < cptr[c + 1] * bs; p++) colour_of[p] = k;
            }
        }
        WfLayout<VT> L;
        if (!make_wf_layout(L, upper != 0, N, val, cind, rptr, colours, bs, colour_of.data(), (size_t)1 << 30,
                            rowmap))
            return fail("layout does not fit");
        const int ng = (int)L.groups.size();
        const size_t nslots = L.col.size();
        std::vector<int> owner(N, -1), done(N, 0);
        for (int g = 0; g < ng; g++)
            for (int q = 0; q < L.groups[g].nchains; q++)
                for (int l = 0; l < bs; l++) {
                    const int r = L.chains[(size_t)g * 32 + q].x + l;
                    if (r < 0 || r >= N) return fail("chain row out of range");
                    if (owner[r] >= 0) return fail("row in two chains");
                    owner[r] = g;
                }
        for (int r = 0; r < N; r++)
            if (owner[r] < 0) return fail("row not in any chain");
        std::vector<VT> yy(x, x + N);  // in place, as the plan's U sweep runs
        for (int g = 0; g < ng; g++) {
            const WfGroup d = L.groups[g];
            const int slots = d.emax + d.imax;
            if (slots > L.slots_max) return fail("group block larger than the warp's buffer");
            if (d.off < 0 || (size_t)d.off + (size_t)slots * 32 > nslots) return fail("group block out of range");
            if (d.off % 4) return fail("group block not 16-byte aligned");
            std::set<int> deps(L.dep_idx.begin() + L.dep_ptr[g], L.dep_idx.begin() + L.dep_ptr[g + 1]);
            for (int dg : deps)
                if (dg < 0 || dg >= g) return fail("dependency not earlier");
            // the staged block
            const int *cw = L.col.data() + d.off;
            const VT *vw = L.val.data() + d.off;
            for (int lane = 0; lane < 32; lane++) {
                bool par_check = false;
                const bool live = lane < d.nchains;
                const int2 ch = L.chains[(size_t)g * 32 + lane];
                if (!live) continue;
                const int r0 = ch.x, E = ch.y & 0xffff, I = (int)((unsigned)ch.y >> 16);
                if (E > d.emax || I > d.imax) return fail("chain count above the group's width");
                // per-row counts as the CTA-per-group kernel reads them: row l's
                // external entries start after those of the rows before it in
                // solve order, and each carries row l in its word
                const unsigned char *cq = L.counts.data() + ((size_t)g * 32 + lane) * 2 * bs;
                int esum = 0, isum = 0;
                for (int l = 0; l < bs; l++) {
                    int eo = 0;
                    for (int r = 0; r < bs; r++)
                        if (upper ? r > l : r < l) eo += cq[r];
                    for (int k = 0; k < cq[l]; k++) {
                        const size_t at = (size_t)(eo + k) * 32 + lane;
                        if (at >= (size_t)d.emax * 32) return fail("row offset beyond the external slots");
                        if ((int)((unsigned)cw[at] >> kColBits) != l) return fail("row count points at another row");
                    }
                    esum += cq[l];
                    isum += cq[bs + l];
                }
                if (esum != E || isum != I) return fail("row counts do not add up to the chain's counts");
                // the lane-per-row form of the in-chain recurrence (k_sweep_cc)
                // is checked against the sequential walk below: tsh_par holds
                // its result, computed from the same phase-1 values
                par_check = true;
                std::vector<VT> tsh(bs), dsh(bs);
                for (int l = 0; l < bs; l++) {
                    tsh[l] = yy[r0 + l];
                    if (upper) dsh[l] = L.dinv[r0 + l];
                }
                VT t = 0;
                int cur = -1;
                for (int e = 0; e < E; e++) {
                    const size_t at = (size_t)e * 32 + lane;
                    if (at >= (size_t)slots * 32) return fail("external slot out of block");
                    const int w = cw[at];
                    const int c = w & kColMask, r = (int)((unsigned)w >> kColBits);
                    if (c < 0 || c >= N) return fail("gather out of range");
                    if (!done[c]) return fail("gather of an unfinished row");
                    if (!deps.count(owner[c])) return fail("gathered row's group not a dependency");
                    if (r < 0 || r >= bs) return fail("row out of chain");
                    if (r != cur) {
                        if (cur >= 0) tsh[cur] = t;
                        cur = r;
                        t = tsh[r];
                    }
                    t -= vw[at] * yy[c];
                }
                if (cur >= 0) tsh[cur] = t;
                // in-chain entries of this lane start after those of the lanes before it
                int ibase = 0;
                for (int q2 = 0; q2 < lane; q2++) ibase += (int)((unsigned)L.chains[(size_t)g * 32 + q2].y >> 16);
                std::vector<VT> tsh_par(tsh);
                if (par_check) {
                    // lane rr keeps its next two in-chain entries; step s finishes
                    // column c and every lane whose next entry is c uses it
                    std::vector<int> left(bs), at(bs), c0(bs, -1), c1(bs, -1);
                    std::vector<VT> v0(bs, 0), v1(bs, 0);
                    const int *iw = cw + (size_t)d.emax * 32 + ibase;
                    const VT *iv = vw + (size_t)d.emax * 32 + ibase;
                    for (int rr = 0; rr < bs; rr++) {
                        int io = 0;
                        for (int r = 0; r < bs; r++)
                            if (upper ? r > rr : r < rr) io += cq[bs + r];
                        left[rr] = cq[bs + rr];
                        at[rr] = io;
                        if (left[rr] > 0) { c0[rr] = iw[at[rr]] & 255; v0[rr] = iv[at[rr]]; at[rr]++; }
                        if (left[rr] > 1) { c1[rr] = iw[at[rr]] & 255; v1[rr] = iv[at[rr]]; at[rr]++; }
                    }
                    for (int s = 0; s < bs; s++) {
                        const int c = upper ? bs - 1 - s : s;
                        if (upper) tsh_par[c] *= dsh[c];
                        const VT yc = tsh_par[c];
                        for (int rr = 0; rr < bs; rr++) {
                            if (rr == c || c0[rr] != c) continue;
                            tsh_par[rr] -= v0[rr] * yc;
                            left[rr]--;
                            c0[rr] = c1[rr];
                            v0[rr] = v1[rr];
                            c1[rr] = -1;
                            if (left[rr] > 1) {
                                if (at[rr] >= I) return fail("in-chain window beyond the chain's entries");
                                c1[rr] = iw[at[rr]] & 255;
                                v1[rr] = iv[at[rr]];
                                at[rr]++;
                            }
                        }
                    }
                    for (int rr = 0; rr < bs; rr++)
                        if (left[rr] != 0) return fail("lane-per-row recurrence left entries unused");
                }
                int e = 0;
                for (int s = 0; s < bs; s++) {
                    const int r = upper ? bs - 1 - s : s;
                    VT tt = tsh[r];
                    while (e < I) {
                        const size_t at = (size_t)d.emax * 32 + ibase + e;
                        if (at >= (size_t)slots * 32) return fail("in-chain slot out of block");
                        const int w = cw[at];
                        if ((w >> 8) != r) break;
                        const int c = w & 255;
                        if (c < 0 || c >= bs) return fail("in-chain column out of chain");
                        if (upper ? c <= r : c >= r) return fail("in-chain column not solved before its row");
                        tt -= vw[at] * tsh[c];
                        e++;
                    }
                    if (upper) tt *= dsh[r];
                    tsh[r] = tt;
                }
                if (e != I) return fail("in-chain entries left over");
                for (int r = 0; r < bs; r++)
                    if (tsh_par[r] != tsh[r]) return fail("lane-per-row recurrence differs from the sequential one");
                for (int l = 0; l < bs; l++) yy[r0 + l] = tsh[l];
            }
            for (int lane = 0; lane < d.nchains; lane++)
                for (int l = 0; l < bs; l++) done[L.chains[(size_t)g * 32 + lane].x + l] = 1;
        }
        std::memcpy(y, yy.data(), sizeof(VT) * N);
        return 0;
    } catch (const std::exception &ex) {
        return fail(ex.what());
    }
}

// The schedule of the cooperative sweep (k_sweep_cp) on `grid` CTAs, repeated
// on the CPU: each CTA's walk over the colours (first_from / next group), the
// group it stages into each of its two buffers and when it consumes it, with
// the staged bytes checked against the buffer size the host computes (the
// widest colour's block plus the row counts, rounded to 128 bytes) and the
// copy addresses and sizes against TMA's 16-byte rule. Every group must be
// solved exactly once, by the CTA the kernel assigns, after that CTA's groups
// of the colours before its own (the grid barriers order the other CTAs').
template <typename VT>
int cp_schedule(int N, const VT *val, const int *cind, const int *rptr, int upper, const int *cptr, int cnum, int bs,
                int grid, char *err, int errlen)
{
    auto fail = [&](const std::string &m) {
        std::snprintf(err, errlen, "%s", m.c_str());
        return 1;
    };
    try {
        std::vector<WfColour> colours;
        std::vector<int> colour_of(N);
        for (int k = 0; k < cnum; k++) {
            const int c = upper ? cnum - 1 - k : k;
            colours.push_back({cptr[c] * bs, cptr[c + 1] * bs});
            for (int p = cptr[c] * bs; p < cptr[c + 1] * bs; p++) colour_of[p] = k;
        }
        WfLayout<VT> L;
        if (!make_wf_layout(L, upper != 0, N, val, cind, rptr, colours, bs, colour_of.data(), (size_t)160 * 1024))
            return fail("layout does not fit");
        const std::vector<int> &cg = L.colour_groups;
        const int nc = (int)cg.size() - 1;
        size_t buf = 0;  // as the host: per colour, widest block + counts, 16-byte rounded; then 128
        for (int c = 0; c < nc; c++)
            buf = std::max(buf, ((size_t)L.colour_slots[c] * 32 * (4 + sizeof(VT)) + 32 * 2 * (size_t)bs + 15) / 16 * 16);
        buf = (buf + 127) / 128 * 128;
        const size_t nbytes = 32 * 2 * (size_t)bs;
        if (buf % 16 || nbytes % 16) return fail("buffer or count block not a multiple of 16 bytes");
        std::vector<int> solved((size_t)cg[nc], 0);
        int widest = 0;
        for (int c = 0; c < nc; c++) widest = std::max(widest, cg[c + 1] - cg[c]);
        if (grid > widest) return fail("grid wider than the widest colour");
        for (int b = 0; b < grid; b++) {
            auto first_from = [&](int c, int *cc) {
                for (; c < nc; c++)
                    if (cg[c] + b < cg[c + 1]) {
                        *cc = c;
                        return cg[c] + b;
                    }
                return -1;
            };
            int staged[2] = {-1, -1};
            auto stage = [&](int g, int k) {
                if (staged[k] >= 0) return fail("buffer restaged before its group was solved");
                const WfGroup &d = L.groups[g];
                const size_t slots = (size_t)d.emax + d.imax;
                const size_t cb = slots * 32 * 4, vb = slots * 32 * sizeof(VT);
                if (cb + vb + nbytes > buf) return fail("group block larger than the staging buffer");
                if ((size_t)d.off % 32 || cb % 16 || vb % 16) return fail("copy not 16-byte aligned");
                if ((size_t)d.off + slots * 32 > L.col.size()) return fail("block past the factor");
                if ((size_t)(g + 1) * nbytes > L.counts.size()) return fail("counts past the array");
                staged[k] = g;
                return 0;
            };
            int k = 0, cd = 0;
            int g0 = first_from(0, &cd);
            if (g0 < 0) return fail("a CTA without a group");
            if (stage(g0, 0)) return 1;
            for (int c = 0; c < nc; c++) {
                const int ge = cg[c + 1];
                for (int g = cg[c] + b; g < ge; g += grid) {
                    int cn = c, gn = g + grid;
                    if (gn >= ge) gn = first_from(c + 1, &cn);
                    if (staged[k] != g) return fail("solved group is not the one staged in its buffer");
                    staged[k] = -1;
                    if (gn >= 0 && stage(gn, k ^ 1)) return 1;
                    for (int cc = 0; cc < c; cc++)
                        for (int h = cg[cc]; h < cg[cc + 1]; h++)
                            if (!solved[h] && (h - cg[cc]) % grid == b) return fail("earlier colour not finished");
                    solved[g]++;
                    k ^= 1;
                }
            }
            if (staged[0] >= 0 || staged[1] >= 0) return fail("a staged group was never solved");
        }
        for (size_t g = 0; g < solved.size(); g++)
            if (solved[g] != 1) return fail("group " + std::to_string(g) + " solved " + std::to_string(solved[g]) + " times");
        return 0;
    } catch (const std::exception &ex) {
        return fail(ex.what());
    }
}

}  // namespace

// The row-per-lane sweep (k_sweep_rl) on the chain-major layout, repeated on
// the CPU with every index checked: lane rr of chain q takes row rr; its
// external entries are the chain's stream at q*emax from the prefix of the
// external counts of the rows before it (L) or after it (U), its in-chain
// entries start at the descriptor's offset (ibase, high half of .y) plus the
// same prefix of the in-chain counts; the recurrence runs bs - 1 steps in
// lockstep over the chain's lanes, a step's column broadcast from its lane
// (U: the value times the inverted diagonal), each lane subtracting it when
// the column's bit is in its mask.
template <typename VT>
int emulate_rl(int N, const VT *val, const int *cind, const int *rptr, int upper, const int *cptr, int cnum, int bs,
               const VT *x, VT *y, char *err, int errlen)
{
    auto fail = [&](const std::string &m) {
        std::snprintf(err, errlen, "%s", m.c_str());
        return 1;
    };
    try {
        std::vector<WfColour> colours;
        std::vector<int> colour_of(N);
        for (int k = 0; k < cnum; k++) {
            const int c = upper ? cnum - 1 - k : k;
            colours.push_back({cptr[c] * bs, cptr[c + 1] * bs});
            for (int p = cptr[c] * bs; p < cptr[c + 1] * bs; p++) colour_of[p] = k;
        }
        WfLayout<VT> L;
        if (!make_wf_layout(L, upper != 0, N, val, cind, rptr, colours, bs, colour_of.data(), (size_t)1 << 30,
                            nullptr, true))
            return fail("layout does not fit");
        std::vector<int> done(N, 0);
        std::vector<VT> yy(x, x + N);
        std::vector<int> fin;  // rows the current colour finishes: readable once it ends
        for (size_t col = 0; col + 1 < L.colour_groups.size(); col++) {
            for (int g = L.colour_groups[col]; g < L.colour_groups[col + 1]; g++) {
                const WfGroup d = L.groups[g];
                if (d.emax > 0 && d.emax % 2 == 0) return fail("chain-major stride not odd");
                const size_t slots = (size_t)d.emax + d.imax;
                if ((size_t)d.off + slots * 32 > L.col.size()) return fail("block beyond the layout");
                const int *cw = L.col.data() + d.off;
                const VT *vw = L.val.data() + d.off;
                for (int q = 0; q < d.nchains; q++) {
                    const int2 cd = L.chains[(size_t)g * 32 + q];
                    const int r0 = cd.x, ibase = (int)((unsigned)cd.y >> 16);
                    const unsigned char *cq = L.counts.data() + ((size_t)g * 32 + q) * 2 * bs;
                    std::vector<VT> tt(bs), sc(bs), di(bs);
                    std::vector<int> at(bs), left(bs);
                    std::vector<uint32_t> mask(bs, 0);
                    for (int rr = 0; rr < bs; rr++) {
                        int eo = 0, io = 0;
                        for (int r = 0; r < bs; r++)
                            if (upper ? r > rr : r < rr) {
                                eo += cq[r];
                                io += cq[bs + r];
                            }
                        const int ne = cq[rr];
                        left[rr] = cq[bs + rr];
                        VT t = yy[r0 + rr];
                        for (int k = 0; k < ne; k++) {
                            const int e = eo + k;
                            if (e >= d.emax) return fail("external entry beyond the chain's stream");
                            const size_t idx = (size_t)q * d.emax + e;
                            const int w = cw[idx];
                            const int c = w & kColMask, r = (int)((unsigned)w >> kColBits);
                            if (r != rr) return fail("external entry of another row");
                            if (c < 0 || c >= N) return fail("gather out of range");
                            if (!done[c]) return fail("gather of an unfinished row");
                            t -= vw[idx] * yy[c];
                        }
                        at[rr] = ibase + io;
                        for (int k = 0; k < left[rr]; k++) {
                            const size_t idx = (size_t)d.emax * 32 + at[rr] + k;
                            if (idx >= slots * 32) return fail("in-chain entry beyond the block");
                            const int w = cw[idx];
                            if ((w >> 8) != rr) return fail("in-chain entry of another row");
                            const int c = w & 255;
                            if (c < 0 || c >= bs || (upper ? c <= rr : c >= rr)) return fail("in-chain column out of order");
                            mask[rr] |= 1u << c;
                        }
                        tt[rr] = t;
                        di[rr] = upper ? L.dinv[r0 + rr] : VT(1);
                        sc[rr] = tt[rr] * di[rr];
                    }
                    const int end_ib = ibase + [&] {
                        int s = 0;
                        for (int r = 0; r < bs; r++) s += cq[bs + r];
                        return s;
                    }();
                    for (int s = 0; s < bs - 1; s++) {
                        const int c = upper ? bs - 1 - s : s;
                        const VT yc = upper ? sc[c] : tt[c];
                        for (int rr = 0; rr < bs; rr++) {
                            if (!(mask[rr] & (1u << c))) continue;
                            if (at[rr] >= end_ib) return fail("in-chain entries of the next chain");
                            tt[rr] -= vw[(size_t)d.emax * 32 + at[rr]] * yc;
                            at[rr]++;
                            if (upper) sc[rr] = tt[rr] * di[rr];
                        }
                    }
                    for (int rr = 0; rr < bs; rr++) {
                        int io = 0;
                        for (int r = 0; r < bs; r++)
                            if (upper ? r > rr : r < rr) io += cq[bs + r];
                        if (at[rr] != ibase + io + left[rr]) return fail("in-chain entries left unused");
                        yy[r0 + rr] = upper ? sc[rr] : tt[rr];
                        fin.push_back(r0 + rr);
                    }
                }
            }
            // the groups of a colour run at once: its rows are readable when it ends
            for (int r : fin) done[r] = 1;
            fin.clear();
        }
        std::memcpy(y, yy.data(), sizeof(VT) * N);
        return 0;
    } catch (const std::exception &ex) {
        return fail(ex.what());
    }
}

extern "C" int wf_emulate_d(int N, const double *val, const int *cind, const int *rptr, int upper, const int *cptr,
                            int cnum, int bs, const double *x, double *y, char *err, int errlen)
{
    return emulate<double>(N, val, cind, rptr, upper, cptr, cnum, bs, x, y, err, errlen);
}

extern "C" int wf_emulate_levels_d(int N, const double *val, const int *cind, const int *rptr, int upper,
                                   const int *levptr, int nlev, const int *rowmap, const double *x, double *y,
                                   char *err, int errlen)
{
    return emulate<double>(N, val, cind, rptr, upper, levptr, nlev, 1, x, y, err, errlen, rowmap);
}

extern "C" int wf_emulate_s(int N, const float *val, const int *cind, const int *rptr, int upper, const int *cptr,
                            int cnum, int bs, const float *x, float *y, char *err, int errlen)
{
    return emulate<float>(N, val, cind, rptr, upper, cptr, cnum, bs, x, y, err, errlen);
}

extern "C" int wf_cp_schedule_s(int N, const float *val, const int *cind, const int *rptr, int upper, const int *cptr,
                                int cnum, int bs, int grid, char *err, int errlen)
{
    return cp_schedule<float>(N, val, cind, rptr, upper, cptr, cnum, bs, grid, err, errlen);
}

extern "C" int wf_cp_schedule_d(int N, const double *val, const int *cind, const int *rptr, int upper,
                                const int *cptr, int cnum, int bs, int grid, char *err, int errlen)
{
    return cp_schedule<double>(N, val, cind, rptr, upper, cptr, cnum, bs, grid, err, errlen);
}

extern "C" int wf_emulate_rl_d(int N, const double *val, const int *cind, const int *rptr, int upper, const int *cptr,
                               int cnum, int bs, const double *x, double *y, char *err, int errlen)
{
    return emulate_rl<double>(N, val, cind, rptr, upper, cptr, cnum, bs, x, y, err, errlen);
}

extern "C" int wf_emulate_rl_s(int N, const float *val, const int *cind, const int *rptr, int upper, const int *cptr,
                               int cnum, int bs, const float *x, float *y, char *err, int errlen)
{
    return emulate_rl<float>(N, val, cind, rptr, upper, cptr, cnum, bs, x, y, err, errlen);
}
