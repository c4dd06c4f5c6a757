#pragma once
// ILU sweep plans: the split factors re-laid out for triangular sweeps on the
// GPU (replaces include/senk_sparse.hpp:132-315, SptrsvCsr_l/_u in their
// sequential, AMC and ABMC forms).
//
// Two layouts. Both take chains (`bs` consecutive schedule positions, one ABMC
// block, solved in order) 32 at a time from one colour, and keep each row's
// subtraction order (entries of other chains first, which are final before the
// colour starts, then in-chain entries; each part in the reference's column
// order: ascending for L, descending for U).
//  * Compact chains (default for AMC/ABMC schedules, `k_sweep_wf`, one launch
//    per sweep, one warp per group of 32 chains): each chain's entries are
//    packed one after another, lane = chain, so a group pads only to its widest
//    chain; the chains of a colour are sorted by their entry counts first.
//  * Row slots (`k_sweep`, one launch per colour; level-set schedules of the
//    natural order, and SENK_SWEEP_COLOURS): slot k of row l of every chain of
//    a group is one 32-wide column, rows padded to the group's widest.
#include <algorithm>
#include <climits>
#include <memory>

#include "device.hpp"

namespace senkgpu {

namespace {

struct Group {
    int p0, p1;  // schedule positions [p0, p1)
};

template <typename VT>
void build_factor(SweepFactor<VT> &F, bool upper, int N, const VT *val, const int *cind, const int *rptr,
                  const std::vector<Group> &groups, const std::vector<int> *rowmap, int bs,
                  const std::vector<int> *group_of_row, cudaStream_t s)
{
    F.upper = upper;
    F.mapped = rowmap != nullptr;
    F.bs = bs;
    const bool chains = !F.mapped && bs > 1;
    std::vector<int> next(N), nint(N);
    int bad = -1;
#pragma omp parallel for schedule(static)
    for (int p = 0; p < N; p++) {
        const int row = rowmap ? (*rowmap)[p] : p;
        int b = rptr[row], e = rptr[row + 1];
        bool ok = true;
        if (upper) {
            ok = e > b && cind[b] == row;  // U row must start with its diagonal
            b++;
        }
        const int cs = row - row % bs, ce = cs + bs;
        int ni = 0;
        for (int j = b; j < e && ok; j++) {
            const int c = cind[j];
            if (c < 0 || c >= N || (upper ? c <= row : c >= row)) { ok = false; break; }
            if (chains && c >= cs && c < ce) ni++;
            else if (group_of_row && (*group_of_row)[c] >= (*group_of_row)[row])
                ok = false;  // a column outside the chain must belong to a group solved earlier
        }
        if (!ok || e - b - ni > 255 || ni > 255) {
#pragma omp atomic write
            bad = row;
        }
        next[p] = (e - b) - ni;
        nint[p] = ni;
    }
    SENK_REQUIRE(bad < 0, std::string(upper ? "U" : "L") + " factor row " + std::to_string(bad) +
                              " does not fit the schedule (diagonal first in U, strictly triangular, "
                              "columns of other chains in earlier colours, at most 255 entries)");
    // Groups of up to 32 chains inside each colour, in processing order.
    std::vector<GroupDesc> gd;
    F.colour_groups.assign(1, 0);
    for (const Group &g : groups) {
        const int nch = (g.p1 - g.p0) / bs;
        for (int q = 0; q < nch; q += 32) {
            GroupDesc d{};
            d.pos0 = g.p0 + q * bs;
            d.nchains = std::min(32, nch - q);
            d.widx = (int)gd.size() * 2 * bs;
            gd.push_back(d);
        }
        F.colour_groups.push_back((int)gd.size());
    }
    const int ng = (int)gd.size();
    std::vector<unsigned char> wd((size_t)std::max(ng, 1) * 2 * bs, 0);
    std::vector<long long> slots(ng, 0);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < ng; i++) {
        long long tot = 0;
        for (int l = 0; l < bs; l++) {
            int we = 0, wi = 0;
            for (int q = 0; q < gd[i].nchains; q++) {
                const int p = gd[i].pos0 + q * bs + l;
                we = std::max(we, next[p]);
                wi = std::max(wi, nint[p]);
            }
            wd[(size_t)gd[i].widx + l] = (unsigned char)we;
            wd[(size_t)gd[i].widx + bs + l] = (unsigned char)wi;
            tot += we + wi;
        }
        slots[i] = tot;
    }
    long long off = 0;
    for (int i = 0; i < ng; i++) {
        gd[i].off = (int)off;
        off += slots[i] * 32;
        SENK_REQUIRE(off < INT_MAX, "factor too large for 32-bit slot offsets");
    }
    // Shared memory a colour's CTAs need to stage their group's block.
    F.colour_smem.assign(F.colour_groups.size() - 1, 0);
    for (size_t c = 0; c + 1 < F.colour_groups.size(); c++)
        for (int i = F.colour_groups[c]; i < F.colour_groups[c + 1]; i++)
            F.colour_smem[c] = std::max(F.colour_smem[c], (size_t)slots[i] * 32 * (sizeof(VT) + sizeof(int)));
    F.elems = off;
    // padding is (0, column -1); filled in parallel (the arrays run to 100s of MB)
    const long long ne = std::max<long long>(off, 1);
    std::unique_ptr<VT[]> hv(new VT[ne]);
    std::unique_ptr<int[]> hc(new int[ne]);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < ne; i++) {
        hv[i] = VT(0);
        hc[i] = -1;
    }
    std::vector<VT> hd(upper ? N : 0);
    long long stored = 0;
#pragma omp parallel for schedule(static) reduction(+ : stored)
    for (int i = 0; i < ng; i++) {
        const GroupDesc d = gd[i];
        const unsigned char *w = wd.data() + d.widx;
        int eoff[32], ioff[32];
        int acc = 0;
        for (int l = 0; l < bs; l++) { eoff[l] = acc; acc += w[l]; }
        for (int l = 0; l < bs; l++) { ioff[l] = acc; acc += w[bs + l]; }
        for (int q = 0; q < d.nchains; q++) {
            for (int l = 0; l < bs; l++) {
                const int p = d.pos0 + q * bs + l;
                const int row = rowmap ? (*rowmap)[p] : p;
                const int cs = row - row % bs, ce = cs + bs;
                int ke = 0, ki = 0;
                auto put = [&](int j) {
                    const int c = cind[j];
                    long long at;
                    if (chains && c >= cs && c < ce) {
                        at = d.off + (long long)(ioff[l] + ki++) * 32 + q;
                        hc[at] = c - cs;
                    } else {
                        at = d.off + (long long)(eoff[l] + ke++) * 32 + q;
                        hc[at] = c;
                    }
                    hv[at] = val[j];
                    stored++;
                };
                if (upper) {
                    hd[p] = val[rptr[row]];
                    for (int j = rptr[row + 1] - 1; j >= rptr[row] + 1; j--) put(j);
                } else {
                    for (int j = rptr[row]; j < rptr[row + 1]; j++) put(j);
                }
            }
        }
    }
    F.nnz = stored + (upper ? N : 0);
    F.val.alloc(ne);
    F.val.upload(hv.get(), ne, s);
    F.col.alloc(ne);
    F.col.upload(hc.get(), ne, s);
    if (upper) {
        F.dinv.alloc(N);
        F.dinv.upload(hd.data(), N, s);
    }
    if (rowmap) {
        F.rowmap.alloc(N);
        F.rowmap.upload(rowmap->data(), N, s);
    }
    F.groups.alloc(std::max(ng, 1));
    F.groups.upload(gd.data(), ng, s);
    F.widths.alloc(wd.size());
    F.widths.upload(wd.data(), wd.size(), s);
    F.dataflow = false;
    F.compact = false;
    F.persistent = false;
    F.force_wide = false;
    F.rowlane = false;
    // Host vectors are released on return: finish the copies first.
    SENK_CUDA(cudaStreamSynchronize(s));
}

// Largest block staged through shared memory; bigger groups read the factor
// from global memory instead.
constexpr size_t kMaxStagedBytes = 160 * 1024;

// Largest dynamic shared memory of one dataflow CTA.
constexpr size_t kMaxWfSmem = 200 * 1024;

// Largest vector the single-CTA sweeps of small systems keep in shared memory,
// and the most dynamic shared memory of that kernel (vector + two staging
// buffers).
constexpr size_t kSmallBytes = 192 * 1024;
constexpr size_t kSmallSmem = 220 * 1024;

// Compact chain layout (wf_layout.hpp) uploaded for k_sweep_wf. Returns false
// (and builds nothing) when a group's block would not fit one warp's shared
// memory; the caller then takes the row-slot layout.
template <typename VT>
bool build_factor_wf(SweepFactor<VT> &F, bool upper, int N, const VT *val, const int *cind, const int *rptr,
                     const std::vector<Group> &colours, int bs, const std::vector<int> &colour_of, bool dataflow,
                     cudaStream_t s, const std::vector<int> *rowmap = nullptr, bool chain_major = false)
{
    std::vector<WfColour> cr;
    for (const Group &g : colours) cr.push_back({g.p0, g.p1});
    WfLayout<VT> lay;
    if (!make_wf_layout(lay, upper, N, val, cind, rptr, cr, bs, colour_of.data(),
                        dataflow ? kMaxWfSmem : kMaxStagedBytes, rowmap ? rowmap->data() : nullptr, chain_major))
        return false;
    const int ng = (int)lay.groups.size();
    F.launches.clear();
    F.upper = upper;
    F.mapped = false;
    F.bs = bs;
    F.compact = true;
    F.dataflow = dataflow;
    F.persistent = false;
    F.force_wide = false;
    F.rowlane = chain_major;
    F.ngroups = ng;
    F.slots_max = lay.slots_max;
    F.elems = (long long)lay.col.size();
    F.nnz = lay.stored + (upper ? N : 0);
    F.colour_groups = lay.colour_groups;
    F.colour_slots = lay.colour_slots;
    F.colour_smem.assign(F.colour_slots.size(), 0);
    F.val.alloc(std::max<size_t>(lay.val.size(), 1));
    F.val.upload(lay.val.data(), lay.val.size(), s);
    F.col.alloc(std::max<size_t>(lay.col.size(), 1));
    F.col.upload(lay.col.data(), lay.col.size(), s);
    if (upper) {
        F.dinv.alloc(N);
        F.dinv.upload(lay.dinv.data(), N, s);
    }
    F.wgroups.alloc(std::max(ng, 1));
    F.wgroups.upload(lay.groups.data(), ng, s);
    F.wchains.alloc(std::max<size_t>(lay.chains.size(), 1));
    F.wchains.upload(lay.chains.data(), lay.chains.size(), s);
    F.wcounts.alloc(std::max<size_t>(lay.counts.size(), 16));
    F.wcounts.upload(lay.counts.data(), lay.counts.size(), s);
    F.dcolour_groups.alloc(lay.colour_groups.size());
    F.dcolour_groups.upload(lay.colour_groups.data(), lay.colour_groups.size(), s);
    std::vector<int4> lv;
    for (size_t c = 0; c + 1 < lay.colour_groups.size(); c++) {
        const int g0 = lay.colour_groups[c], g1 = lay.colour_groups[c + 1];
        int e0 = 0, ne = 0;
        if (g1 > g0) {
            const WfGroup &last = lay.groups[g1 - 1];
            e0 = lay.groups[g0].off;
            ne = last.off + (last.emax + last.imax) * 32 - e0;
        }
        lv.push_back(make_int4(g0, g1 - g0, e0, ne));
    }
    F.levels.alloc(std::max<size_t>(lv.size(), 1));
    F.levels.upload(lv.data(), lv.size(), s);
    if (upper) {
        F.cdinv.alloc(std::max<size_t>(lay.cdinv.size(), 1));
        F.cdinv.upload(lay.cdinv.data(), lay.cdinv.size(), s);
    }
    F.level_bytes = 0;
    for (size_t c = 0; c + 1 < lay.colour_groups.size(); c++) {
        const int G = lay.colour_groups[c + 1] - lay.colour_groups[c];
        long long ne = 0;
        for (int g = lay.colour_groups[c]; g < lay.colour_groups[c + 1]; g++)
            ne += (long long)(lay.groups[g].emax + lay.groups[g].imax) * 32;
        const size_t b = (size_t)G * 16 + (size_t)G * 256 + (size_t)ne * (4 + sizeof(VT)) +
                         (upper ? (size_t)G * 32 * bs * sizeof(VT) : 0);
        F.level_bytes = std::max(F.level_bytes, b);
    }
    if (!dataflow) {
        // one launch per colour; x is read early from the second colour on
        const int nc = (int)lay.colour_groups.size() - 1;
        for (int c = 0; c < nc; c++) {
            typename SweepFactor<VT>::Launch L{};
            L.g0 = lay.colour_groups[c];
            L.g1 = lay.colour_groups[c + 1];
            L.early_x = c > 0 ? 1 : 0;
            L.smem = ((size_t)lay.colour_slots[c] * 32 * (4 + sizeof(VT)) + 32 * 2 * (size_t)bs + 15) / 16 * 16;
            if (L.g1 > L.g0) F.launches.push_back(L);
        }
    } else {
        F.dep_ptr.alloc(lay.dep_ptr.size());
        F.dep_ptr.upload(lay.dep_ptr.data(), lay.dep_ptr.size(), s);
        F.dep_idx.alloc(std::max<size_t>(lay.dep_idx.size(), 1));
        F.dep_idx.upload(lay.dep_idx.data(), lay.dep_idx.size(), s);
        F.flags.alloc(std::max(ng, 1));
        SENK_CUDA(cudaMemsetAsync(F.flags.p, 0, F.flags.bytes(), s));
        const int ctrl0[4] = {0, 1, 0, 0};  // counter, epoch, abort, warps finished
        F.ctrl.alloc(4);
        F.ctrl.upload(ctrl0, 4, s);
    }
    SENK_CUDA(cudaStreamSynchronize(s));  // the layout's host arrays are released on return
    return true;
}

// Level sets of a triangular factor for the natural order: level(i) = 1 + max
// level of the rows it reads. Rows of one level are independent, and each row's
// arithmetic is the sequential sweep's, so the result equals the sequential one.
void level_schedule(int N, const int *cind, const int *rptr, bool upper, std::vector<int> &rowmap,
                    std::vector<Group> &groups)
{
    std::vector<int> lev(N, 0);
    int maxlev = 0;
    if (!upper) {
        for (int i = 0; i < N; i++) {
            int l = 0;
            for (int j = rptr[i]; j < rptr[i + 1]; j++) l = std::max(l, lev[cind[j]] + 1);
            lev[i] = l;
            maxlev = std::max(maxlev, l);
        }
    } else {
        for (int i = N - 1; i >= 0; i--) {
            int l = 0;
            for (int j = rptr[i] + 1; j < rptr[i + 1]; j++) l = std::max(l, lev[cind[j]] + 1);
            lev[i] = l;
            maxlev = std::max(maxlev, l);
        }
    }
    std::vector<int> cnt(maxlev + 2, 0);
    for (int i = 0; i < N; i++) cnt[lev[i] + 1]++;
    for (int l = 0; l <= maxlev; l++) cnt[l + 1] += cnt[l];
    rowmap.assign(N, 0);
    std::vector<int> at(cnt.begin(), cnt.end() - 1);
    for (int i = 0; i < N; i++) rowmap[at[lev[i]]++] = i;
    groups.clear();
    for (int l = 0; l <= maxlev; l++) groups.push_back({cnt[l], cnt[l + 1]});
}


template <typename VT, typename XT, int BS, bool UPPER, bool MAPPED, bool STAGED>
void launch_group(const SweepFactor<VT> &F, int *status, int gb, int ge, size_t smem, const XT *x, XT *y,
                  cudaStream_t s, const int *gate)
{
    auto kern = k_sweep<VT, XT, BS, UPPER, MAPPED, STAGED>;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(ge - gb);
    cfg.blockDim = dim3(BS * 32);
    cfg.dynamicSmemBytes = STAGED ? smem : 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    SENK_CUDA(cudaLaunchKernelEx(&cfg, kern, (const GroupDesc *)F.groups.p, gb, (const unsigned char *)F.widths.p,
                                 (const VT *)F.val.p, (const int *)F.col.p, (const VT *)F.dinv.p,
                                 (const int *)F.rowmap.p, x, y, gate, status));
}

template <typename VT, typename XT, int BS, bool UPPER, bool MAPPED>
void launch_colour(const SweepFactor<VT> &F, int *status, int c, const XT *x, XT *y, cudaStream_t s,
                   const int *gate)
{
    const int gb = F.colour_groups[c], ge = F.colour_groups[c + 1];
    if (ge == gb) return;
    const size_t smem = F.colour_smem[c];
    if (smem <= kMaxStagedBytes) launch_group<VT, XT, BS, UPPER, MAPPED, true>(F, status, gb, ge, smem, x, y, s, gate);
    else launch_group<VT, XT, BS, UPPER, MAPPED, false>(F, status, gb, ge, smem, x, y, s, gate);
}

template <typename VT, typename XT, int BS, bool UPPER, bool MAPPED>
void allow_smem()
{
    SENK_CUDA(cudaFuncSetAttribute(k_sweep<VT, XT, BS, UPPER, MAPPED, true>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxStagedBytes));
}

template <typename VT, typename XT, int BS, bool UPPER>
void launch_wf(const SweepFactor<VT> &F, int *status, const XT *x, XT *y, cudaStream_t s, const int *gate)
{
    if (F.ngroups == 0) return;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(F.wf_grid);
    cfg.blockDim = dim3(F.wf_warps * 32);
    cfg.dynamicSmemBytes = F.wf_smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    SENK_CUDA(cudaLaunchKernelEx(&cfg, k_sweep_wf<VT, XT, BS, UPPER>, (const WfGroup *)F.wgroups.p, 0, F.ngroups,
                                 (const int2 *)F.wchains.p, (const VT *)F.val.p, (const int *)F.col.p,
                                 (const VT *)F.dinv.p, (const int *)F.dep_ptr.p, (const int *)F.dep_idx.p,
                                 F.flags.p, F.ctrl.p, x, y, gate, status, F.slots_max));
}

// Compact chains, one launch per colour (k_sweep_cc), chained by programmatic
// dependent launch.
template <typename VT, typename XT, int BS, bool UPPER>
void launch_cc(const SweepFactor<VT> &F, int *status, const XT *x, XT *y, cudaStream_t s, const int *gate)
{
    for (const auto &L : F.launches) {
        if (L.coop) {
            cudaLaunchConfig_t cfg{};
            cfg.gridDim = dim3(L.grid);
            cfg.blockDim = dim3(BS * 32);
            cfg.dynamicSmemBytes = L.smem;
            cfg.stream = s;
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeCooperative;
            at[0].val.cooperative = 1;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            SENK_CUDA(cudaLaunchKernelEx(&cfg, k_sweep_cp<VT, XT, BS, UPPER>, (const WfGroup *)F.wgroups.p,
                                         (const int *)F.dcolour_groups.p, L.cbeg, L.cend, (const int2 *)F.wchains.p,
                                         (const unsigned char *)F.wcounts.p, (const VT *)F.val.p,
                                         (const int *)F.col.p, (const VT *)F.dinv.p, x, y, gate, status, F.ctrl.p,
                                         (unsigned)F.cp_buf));
            continue;
        }
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3(L.g1 - L.g0);
        cfg.blockDim = dim3(BS * 32);
        cfg.dynamicSmemBytes = L.smem;
        cfg.stream = s;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        if (F.rowlane) {
            if constexpr (BS >= 2) {
                if (L.wide) {
                    cfg.blockDim = dim3(BS * 16);
                    SENK_CUDA(cudaLaunchKernelEx(&cfg, k_sweep_rl<VT, XT, BS, UPPER, 2>, (const WfGroup *)F.wgroups.p,
                                                 L.g0, (const int2 *)F.wchains.p,
                                                 (const unsigned char *)F.wcounts.p, (const VT *)F.val.p,
                                                 (const int *)F.col.p, (const VT *)F.dinv.p, x, y, gate, status,
                                                 L.early_x));
                    continue;
                }
            }
            SENK_CUDA(cudaLaunchKernelEx(&cfg, k_sweep_rl<VT, XT, BS, UPPER, 1>, (const WfGroup *)F.wgroups.p, L.g0,
                                         (const int2 *)F.wchains.p, (const unsigned char *)F.wcounts.p,
                                         (const VT *)F.val.p, (const int *)F.col.p, (const VT *)F.dinv.p, x, y, gate,
                                         status, L.early_x));
            continue;
        }
        if constexpr (BS >= 4) {
            if (L.wide) {
                cfg.blockDim = dim3(BS * 16);
                SENK_CUDA(cudaLaunchKernelEx(&cfg, k_sweep_cc2<VT, XT, BS, UPPER>, (const WfGroup *)F.wgroups.p,
                                             L.g0, (const int2 *)F.wchains.p, (const unsigned char *)F.wcounts.p,
                                             (const VT *)F.val.p, (const int *)F.col.p, (const VT *)F.dinv.p, x, y,
                                             gate, status, L.early_x));
                continue;
            }
        }
        SENK_CUDA(cudaLaunchKernelEx(&cfg, k_sweep_cc<VT, XT, BS, UPPER>, (const WfGroup *)F.wgroups.p, L.g0,
                                     (const int2 *)F.wchains.p, (const unsigned char *)F.wcounts.p,
                                     (const VT *)F.val.p, (const int *)F.col.p, (const VT *)F.dinv.p, x, y, gate,
                                     status, L.early_x));
    }
}

// Dynamic shared memory limits of the per-colour kernels, and which colours
// take the two-rows-per-thread kernel: those with more groups than one wave of
// k_sweep_cc holds at once, when k_sweep_cc2 holds more (or all colours with
// force_wide).
template <typename VT, int BS, bool UPPER>
void shape_cc(SweepFactor<VT> &F)
{
    size_t most = 0;
    for (const auto &L : F.launches) most = std::max(most, L.smem);
    const int lim = (int)std::max<size_t>(most, 48 * 1024);
    if (F.rowlane) {
        SENK_CUDA(cudaFuncSetAttribute(k_sweep_rl<VT, VT, BS, UPPER, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       lim));
        if constexpr (BS >= 2) {
            SENK_CUDA(cudaFuncSetAttribute(k_sweep_rl<VT, VT, BS, UPPER, 2>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, lim));
            for (auto &L : F.launches) {
                if (L.coop) continue;
                if (F.force_wide) {
                    L.wide = 1;
                    continue;
                }
                int one = 0, two = 0;
                SENK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&one, k_sweep_rl<VT, VT, BS, UPPER, 1>,
                                                                        BS * 32, L.smem));
                SENK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&two, k_sweep_rl<VT, VT, BS, UPPER, 2>,
                                                                        BS * 16, L.smem));
                L.wide = (L.g1 - L.g0) > one * sm_count() && two > one ? 1 : 0;
            }
        }
        return;
    }
    SENK_CUDA(cudaFuncSetAttribute(k_sweep_cc<VT, VT, BS, UPPER>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim));
    if constexpr (BS >= 4) {
        SENK_CUDA(cudaFuncSetAttribute(k_sweep_cc2<VT, VT, BS, UPPER>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       lim));
        for (auto &L : F.launches) {
            if (L.coop) continue;
            if (F.force_wide) {
                L.wide = 1;
                continue;
            }
            int one = 0, two = 0;
            SENK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&one, k_sweep_cc<VT, VT, BS, UPPER>, BS * 32,
                                                                    L.smem));
            SENK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&two, k_sweep_cc2<VT, VT, BS, UPPER>, BS * 16,
                                                                    L.smem));
            L.wide = (L.g1 - L.g0) > one * sm_count() && two > one ? 1 : 0;
        }
    }
}

// Shape of the cooperative launches: two staging buffers of the widest group's
// block; as many CTAs fit at once as the occupancy allows. Every run of at
// least two consecutive colours (in processing order) whose groups fit that
// wave becomes one cooperative launch on as many CTAs as its widest colour has
// groups; the other colours keep their own launches. Leaves the launch list
// as it is when the buffers do not fit or the device cannot launch
// cooperatively.
template <typename VT, int BS, bool UPPER>
void shape_cp(SweepFactor<VT> &F)
{
    int coop = 0, dev = 0;
    SENK_CUDA(cudaGetDevice(&dev));
    SENK_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (!coop || F.ngroups == 0) return;
    size_t buf = 0;
    for (const auto &L : F.launches) buf = std::max(buf, L.smem);
    buf = (buf + 127) / 128 * 128;
    if (2 * buf > kMaxWfSmem) return;
    auto kern = k_sweep_cp<VT, VT, BS, UPPER>;
    SENK_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)std::max<size_t>(2 * buf, 48 * 1024)));
    int per_sm = 0;
    SENK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, BS * 32, 2 * buf));
    if (per_sm < 1) return;
    const int wave = per_sm * sm_count();
    const int nc = (int)F.colour_groups.size() - 1;
    auto groups_of = [&](int c) { return F.colour_groups[c + 1] - F.colour_groups[c]; };
    std::vector<typename SweepFactor<VT>::Launch> out;
    int c = 0;
    while (c < nc) {
        int e = c;
        int widest = 0;
        while (e < nc && groups_of(e) <= wave) widest = std::max(widest, groups_of(e++));
        if (e - c >= 2 && widest > 0) {
            typename SweepFactor<VT>::Launch L{};
            L.coop = 1;
            L.cbeg = c;
            L.cend = e;
            L.grid = widest;
            L.smem = 2 * buf;
            out.push_back(L);
            c = e;
            continue;
        }
        if (groups_of(c) > 0) {
            for (const auto &L : F.launches)
                if (L.g0 == F.colour_groups[c]) out.push_back(L);
        }
        c++;
    }
    F.launches = out;
    F.cp_buf = buf;
    if (F.ctrl.n < 4) F.ctrl.alloc(4);
    SENK_CUDA(cudaMemset(F.ctrl.p, 0, 4 * sizeof(int)));
}

// Launch shape of a dataflow sweep: as many warps per CTA (up to 8) as the
// shared memory allows, and as many CTAs as are resident at once (every warp
// loops over groups, so the grid need not cover them).
template <typename VT, int BS, bool UPPER>
void shape_wf(SweepFactor<VT> &F)
{
    auto kern = k_sweep_wf<VT, VT, BS, UPPER>;
    const size_t per_warp = wf_warp_bytes<VT, VT, BS, UPPER>(F.slots_max);
    int warps = (int)std::min<size_t>(8, kMaxWfSmem / per_warp);
    SENK_REQUIRE(warps >= 1, "a group's block exceeds the shared memory of the dataflow sweep");
    warps = std::min(warps, std::max(1, F.ngroups));
    F.wf_warps = warps;
    F.wf_smem = per_warp * warps;
    SENK_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)F.wf_smem));
    int per_sm = 0;
    SENK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, warps * 32, F.wf_smem));
    SENK_REQUIRE(per_sm >= 1, "the dataflow sweep does not fit an SM");
    const int need = (F.ngroups + warps - 1) / warps;
    F.wf_grid = std::max(1, std::min(need, per_sm * sm_count()));
}

template <typename VT, bool UPPER, int BS>
void shape_compact_bs(SweepFactor<VT> &F)
{
    if (F.dataflow) {
        shape_wf<VT, BS, UPPER>(F);
        return;
    }
    shape_cc<VT, BS, UPPER>(F);
    if (F.persistent) shape_cp<VT, BS, UPPER>(F);
}

template <typename VT, bool UPPER>
void shape_wf_bs(SweepFactor<VT> &F)
{
    switch (F.bs) {
    case 1: shape_compact_bs<VT, UPPER, 1>(F); break;
    case 2: shape_compact_bs<VT, UPPER, 2>(F); break;
    case 4: shape_compact_bs<VT, UPPER, 4>(F); break;
    case 8: shape_compact_bs<VT, UPPER, 8>(F); break;
    case 16: shape_compact_bs<VT, UPPER, 16>(F); break;
    case 32: shape_compact_bs<VT, UPPER, 32>(F); break;
    default: throw ArgError("unsupported chain length");
    }
}

template <typename VT, typename XT, bool UPPER>
void sweep_groups(const SweepFactor<VT> &F, int *status, const XT *x, XT *y, cudaStream_t s, const int *gate)
{
    const int nc = (int)F.colour_groups.size() - 1;
    if (F.compact) {
#define SENK_COMPACT_CASE(BS)                                                      \
    case BS:                                                                       \
        if (F.dataflow) launch_wf<VT, XT, BS, UPPER>(F, status, x, y, s, gate);    \
        else launch_cc<VT, XT, BS, UPPER>(F, status, x, y, s, gate);               \
        break;
        switch (F.bs) {
            SENK_COMPACT_CASE(1) SENK_COMPACT_CASE(2) SENK_COMPACT_CASE(4) SENK_COMPACT_CASE(8)
            SENK_COMPACT_CASE(16) SENK_COMPACT_CASE(32)
        default: throw ArgError("unsupported chain length");
        }
#undef SENK_COMPACT_CASE
        SENK_LAUNCH_CHECK();
        return;
    }
    for (int c = 0; c < nc; c++) {
        if (F.mapped) {
            launch_colour<VT, XT, 1, UPPER, true>(F, status, c, x, y, s, gate);
            continue;
        }
        switch (F.bs) {
        case 1: launch_colour<VT, XT, 1, UPPER, false>(F, status, c, x, y, s, gate); break;
        case 2: launch_colour<VT, XT, 2, UPPER, false>(F, status, c, x, y, s, gate); break;
        case 4: launch_colour<VT, XT, 4, UPPER, false>(F, status, c, x, y, s, gate); break;
        case 8: launch_colour<VT, XT, 8, UPPER, false>(F, status, c, x, y, s, gate); break;
        case 16: launch_colour<VT, XT, 16, UPPER, false>(F, status, c, x, y, s, gate); break;
        case 32: launch_colour<VT, XT, 32, UPPER, false>(F, status, c, x, y, s, gate); break;
        default: throw ArgError("unsupported chain length");
        }
    }
}

template <typename VT, typename XT>
void allow_all_smem()
{
    allow_smem<VT, XT, 1, false, true>(); allow_smem<VT, XT, 1, true, true>();
    allow_smem<VT, XT, 1, false, false>(); allow_smem<VT, XT, 1, true, false>();
    allow_smem<VT, XT, 2, false, false>(); allow_smem<VT, XT, 2, true, false>();
    allow_smem<VT, XT, 4, false, false>(); allow_smem<VT, XT, 4, true, false>();
    allow_smem<VT, XT, 8, false, false>(); allow_smem<VT, XT, 8, true, false>();
    allow_smem<VT, XT, 16, false, false>(); allow_smem<VT, XT, 16, true, false>();
    allow_smem<VT, XT, 32, false, false>(); allow_smem<VT, XT, 32, true, false>();
}

}  // namespace

template <typename VT>
void IluPlan<VT>::sweep_small(int which, const VT *x, VT *y, cudaStream_t s, const int *gate) const
{
    auto mk = [](const SweepFactor<VT> &F) {
        return SmallFactor<VT>{(const WfGroup *)F.wgroups.p, (const int2 *)F.wchains.p, (const VT *)F.val.p,
                               (const int *)F.col.p, (const VT *)F.cdinv.p, (const int4 *)F.levels.p,
                               (int)F.colour_groups.size() - 1};
    };
    const int steps = ((which & 1) ? (int)L.colour_groups.size() - 1 : 0) +
                      ((which & 2) ? (int)U.colour_groups.size() - 1 : 0);
    const size_t smem = small_smem_bytes((size_t)n, sizeof(VT), steps, small_buf, small_nbuf);
    // small_threads consumers and one staging warp
    k_ilu_small<VT, VT><<<1, small_threads + 32, smem, s>>>(mk(L), mk(U), which, x, y, n, gate, status.p,
                                                            (int)small_buf, small_nbuf);
    SENK_LAUNCH_CHECK();
}

// Compact layouts of both factors for k_ilu_small (natural order: level sets,
// one row per chain; AMC/ABMC: the colours). Leaves `small` false when a
// factor does not fit the compact layout, so the caller takes the other paths.
template <typename VT>
void IluPlan<VT>::build_small(int N, const VT *lval, const int *lcind, const int *lrptr, const VT *uval,
                              const int *ucind, const int *urptr, int pckind, const int *cptr, int cnum, int bsize,
                              cudaStream_t s)
{
    small = false;
    std::vector<Group> gl, gu;
    std::vector<int> col_l(N), col_u(N), rml, rmu;
    int bs = 1;
    if (pckind == SENK_PC_ILU) {
        level_schedule(N, lcind, lrptr, false, rml, gl);
        level_schedule(N, ucind, urptr, true, rmu, gu);
        for (size_t k = 0; k < gl.size(); k++)
            for (int p = gl[k].p0; p < gl[k].p1; p++) col_l[rml[p]] = (int)k;
        for (size_t k = 0; k < gu.size(); k++)
            for (int p = gu[k].p0; p < gu[k].p1; p++) col_u[rmu[p]] = (int)k;
    } else {
        if (pckind != SENK_PC_ILU_AMC) return;  // chains of several rows: the per-colour launches
        SENK_REQUIRE(cptr && cnum > 0, "colour pointer missing");
        SENK_REQUIRE(cptr[0] == 0 && (long long)cptr[cnum] * bs == N, "colour pointer does not cover N rows");
        for (int k = 0; k < cnum; k++) {
            SENK_REQUIRE(cptr[k + 1] >= cptr[k], "colour pointer not monotone");
            gl.push_back({cptr[k] * bs, cptr[k + 1] * bs});
            for (int p = cptr[k] * bs; p < cptr[k + 1] * bs; p++) {
                col_l[p] = k;
                col_u[p] = cnum - 1 - k;
            }
        }
        for (int k = cnum - 1; k >= 0; k--) gu.push_back(gl[k]);
    }
    if (!build_factor_wf(L, false, N, lval, lcind, lrptr, gl, bs, col_l, false, s, rml.empty() ? nullptr : &rml))
        return;
    if (!build_factor_wf(U, true, N, uval, ucind, urptr, gu, bs, col_u, false, s, rmu.empty() ? nullptr : &rmu))
        return;
    int most = 32;
    for (const SweepFactor<VT> *F : {&L, &U})
        for (size_t c = 0; c + 1 < F->colour_groups.size(); c++)
            most = std::max(most, (F->colour_groups[c + 1] - F->colour_groups[c]) * 32);
    small_threads = std::min(992, (most + 31) / 32 * 32);
    small_buf = (std::max(L.level_bytes, U.level_bytes) + 127) / 128 * 128;
    // the vector and the descriptors of both factors' levels (one application)
    const int steps = (int)L.colour_groups.size() - 1 + (int)U.colour_groups.size() - 1;
    const size_t fixed = small_smem_bytes((size_t)N, sizeof(VT), steps, 0, 0);
    if (fixed + 2 * small_buf > kSmallSmem) return;  // a level too large to stage next to the vector
    small_nbuf = (int)std::min<size_t>(kSmallMaxBufs, (kSmallSmem - fixed) / std::max<size_t>(small_buf, 128));
    const size_t smem = small_smem_bytes((size_t)N, sizeof(VT), steps, small_buf, small_nbuf);
    SENK_CUDA(cudaFuncSetAttribute(k_ilu_small<VT, VT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    small = true;
}

template <typename VT>
void IluPlan<VT>::build(int N, const VT *lval, const int *lcind, const int *lrptr, const VT *uval,
                        const int *ucind, const int *urptr, int pckind, const int *cptr, int cnum, int bsize,
                        cudaStream_t s, int sweep_mode)
{
    SENK_REQUIRE(sweep_mode == SENK_SWEEP_AUTO || sweep_mode == SENK_SWEEP_COLOURS ||
                     sweep_mode == SENK_SWEEP_DATAFLOW || sweep_mode == SENK_SWEEP_COMPACT ||
                     sweep_mode == SENK_SWEEP_PERSISTENT || sweep_mode == SENK_SWEEP_WIDE ||
                     sweep_mode == SENK_SWEEP_ROWS || sweep_mode == SENK_SWEEP_ROWS_WIDE,
                 "unknown sweep mode");
    SENK_REQUIRE(N > 0, "N must be positive");
    SENK_REQUIRE(lval && lcind && lrptr && uval && ucind && urptr, "null factor array");
    n = N;
    precond = pckind;
    status.alloc(1);
    SENK_CUDA(cudaMemsetAsync(status.p, 0, sizeof(int), s));
    allow_all_smem<VT, VT>();
    // Small systems, default schedule: both sweeps in one CTA with the vector in
    // shared memory (one launch per application instead of one per colour or
    // level set).
    small = sweep_mode == SENK_SWEEP_AUTO && (size_t)N * sizeof(VT) <= kSmallBytes;
    if (small) {
        build_small(N, lval, lcind, lrptr, uval, ucind, urptr, pckind, cptr, cnum, bsize, s);
        if (small) return;
    }
    if (pckind == SENK_PC_ILU) {
        std::vector<int> rm;
        std::vector<Group> gr;
        level_schedule(N, lcind, lrptr, false, rm, gr);
        build_factor(L, false, N, lval, lcind, lrptr, gr, &rm, 1, nullptr, s);
        level_schedule(N, ucind, urptr, true, rm, gr);
        build_factor(U, true, N, uval, ucind, urptr, gr, &rm, 1, nullptr, s);
        return;
    }
    SENK_REQUIRE(pckind == SENK_PC_ILU_AMC || pckind == SENK_PC_ILU_ABMC, "unknown preconditioner kind");
    const int bs = pckind == SENK_PC_ILU_AMC ? 1 : bsize;
    SENK_REQUIRE(bs == 1 || bs == 2 || bs == 4 || bs == 8 || bs == 16 || bs == 32,
                 "ABMC block size must be 1, 2, 4, 8, 16 or 32 on the GPU path (got " + std::to_string(bs) + ")");
    SENK_REQUIRE(cptr && cnum > 0, "colour pointer missing");
    SENK_REQUIRE(cptr[0] == 0 && (long long)cptr[cnum] * bs == N, "colour pointer does not cover N rows");
    std::vector<Group> fwd, bwd;
    std::vector<int> colour_of(N);
    for (int k = 0; k < cnum; k++) {
        SENK_REQUIRE(cptr[k + 1] >= cptr[k], "colour pointer not monotone");
        fwd.push_back({cptr[k] * bs, cptr[k + 1] * bs});
        for (int p = cptr[k] * bs; p < cptr[k + 1] * bs; p++) colour_of[p] = k;
    }
    for (int k = cnum - 1; k >= 0; k--) bwd.push_back(fwd[k]);
    // AUTO, as measured on the 128^3 system: FP32 factors on compact chains
    // with the lanes of a chain holding its rows, one launch per colour
    // (application 0.085 ms, against 0.139 ms with a lane per chain and 0.193
    // ms on row slots), FP64 factors on row slots (0.303 ms against 0.318 ms
    // row-per-lane and 0.405 ms lane-per-chain). COLOURS: row slots; COMPACT:
    // compact chains per colour, a lane per chain; ROWS: a chain's rows in its
    // lanes; DATAFLOW: compact chains, one launch per sweep. A factor whose
    // widest group does not fit shared memory falls back to row slots.
    const bool persistent = sweep_mode == SENK_SWEEP_PERSISTENT;
    const bool rows = sweep_mode == SENK_SWEEP_ROWS || sweep_mode == SENK_SWEEP_ROWS_WIDE ||
                      (sweep_mode == SENK_SWEEP_AUTO && sizeof(VT) == 4);
    const bool wide = sweep_mode == SENK_SWEEP_WIDE || sweep_mode == SENK_SWEEP_ROWS_WIDE;
    const bool compact = sweep_mode == SENK_SWEEP_COMPACT || sweep_mode == SENK_SWEEP_DATAFLOW || persistent || wide ||
                         rows || (sweep_mode == SENK_SWEEP_AUTO && sizeof(VT) == 4);
    const bool df = sweep_mode == SENK_SWEEP_DATAFLOW;
    if (!(compact && build_factor_wf(L, false, N, lval, lcind, lrptr, fwd, bs, colour_of, df, s, nullptr, rows)))
        build_factor(L, false, N, lval, lcind, lrptr, fwd, nullptr, bs, &colour_of, s);
    else {
        L.persistent = persistent;
        L.force_wide = wide;
        shape_wf_bs<VT, false>(L);
    }
    // For U, "earlier" means a later colour: flip the colour numbers.
    for (int p = 0; p < N; p++) colour_of[p] = cnum - 1 - colour_of[p];
    if (!(compact && build_factor_wf(U, true, N, uval, ucind, urptr, bwd, bs, colour_of, df, s, nullptr, rows)))
        build_factor(U, true, N, uval, ucind, urptr, bwd, nullptr, bs, &colour_of, s);
    else {
        U.persistent = persistent;
        U.force_wide = wide;
        shape_wf_bs<VT, true>(U);
    }
}

template <typename VT>
template <typename XT>
void IluPlan<VT>::sweep(const SweepFactor<VT> &F, const XT *x, XT *y, cudaStream_t s, const int *gate) const
{
    if (small) {
        sweep_small(F.upper ? 2 : 1, (const VT *)x, (VT *)y, s, gate);
        return;
    }
    if (F.upper) sweep_groups<VT, XT, true>(F, status.p, x, y, s, gate);
    else sweep_groups<VT, XT, false>(F, status.p, x, y, s, gate);
}

template <typename VT>
long long IluPlan<VT>::apply_bytes() const
{
    const long long vb = sizeof(VT);
    // stored entries: value + column; U diagonal: value only; x read, t written,
    // t read and written again by the in-place U sweep.
    return (L.nnz + (U.nnz - n)) * (vb + 4) + (long long)n * vb + 4LL * n * vb;
}

template <typename VT>
void IluPlan<VT>::check_status(cudaStream_t s) const
{
    int h = 0;
    SENK_CUDA(cudaMemcpyAsync(&h, status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    SENK_CUDA(cudaStreamSynchronize(s));
    if (!h) return;
    // reported once: the next sweep starts clean
    SENK_CUDA(cudaMemsetAsync(status.p, 0, sizeof(int), s));
    SENK_CUDA(cudaStreamSynchronize(s));
    throw CudaError{cudaErrorLaunchTimeout,
                    h == 2 ? "ILU sweep: a TMA copy of a factor block did not complete"
                           : "ILU sweep: a wait for an earlier group's or colour's rows ran out",
                    __FILE__, __LINE__};
}

}  // namespace senkgpu
