// Host construction of the Q2 cell blocks (see cell_blocks.h). Deterministic for any thread
// count: every block is built from its own cells alone, and the offsets come from prefix sums
// over blocks in order.
#include "cell_blocks.h"

#include <omp.h>

#include <algorithm>

#include "common.h"

namespace fgb {

namespace {

// sorted (DoF << 16 | item) keys of the cells at positions [p0, p1); returns the number of
// distinct DoFs
int block_keys(const FemStructure& fs, const std::vector<int32_t>& perm, int p0, int p1, uint64_t* keys) {
    const int m = 27 * (p1 - p0);
    for (int p = p0; p < p1; ++p) {
        const int32_t* cd = fs.cell_dofs.data() + 27 * (size_t)perm[p];
        for (int l = 0; l < 27; ++l) {
            const int item = 27 * (p - p0) + l;
            keys[item] = ((uint64_t)(uint32_t)cd[l] << 16) | (uint64_t)item;
        }
    }
    std::sort(keys, keys + m);
    int d = 0;
    for (int e = 0; e < m; ++e)
        if (e == 0 || (keys[e] >> 16) != (keys[e - 1] >> 16)) ++d;
    return d;
}

// split [p0, p1) into halves until every part holds at most max_dofs DoFs; parts are appended
// in position order with their keys left sorted in `keys` (offset 27 * p)
void split_block(const FemStructure& fs, const std::vector<int32_t>& perm, int p0, int p1, int max_dofs,
                 uint64_t* keys, std::vector<std::pair<int, int>>& parts) {
    const int d = block_keys(fs, perm, p0, p1, keys + 27 * (size_t)p0);
    if (d <= max_dofs || p1 - p0 == 1) {
        parts.push_back({p1, d});
        return;
    }
    const int mid = p0 + (p1 - p0) / 2;
    split_block(fs, perm, p0, mid, max_dofs, keys, parts);
    split_block(fs, perm, mid, p1, max_dofs, keys, parts);
}

}  // namespace

CellBlocks build_cell_blocks(const FemStructure& fs, int cells_per_block, int max_dofs) {
    FGB_REQUIRE(fs.order == 2, "cell blocks are built for Q2 structures");
    FGB_REQUIRE(cells_per_block >= 1 && 27 * cells_per_block <= 65535, "27 x cells per block must fit 16 bits");
    FGB_REQUIRE(max_dofs >= 27 && max_dofs <= 4096, "block DoF limit out of range");
    CellBlocks cb;
    SetupPhases phase("cell blocks build");
    const int nc = fs.n_cells, n = fs.n_dofs;
    cb.n_cells = nc;
    cb.n_dofs = n;
    // cells in ascending order of their interior DoF (lattice index 13)
    std::vector<int32_t> owner(n, -1);
#pragma omp parallel for schedule(static)
    for (int c = 0; c < nc; ++c) owner[fs.cell_dofs[27 * (size_t)c + 13]] = c;
    cb.perm.reserve(nc);
    for (int d = 0; d < n; ++d)
        if (owner[d] >= 0) cb.perm.push_back(owner[d]);
    FGB_REQUIRE((int)cb.perm.size() == nc, "every cell owns one interior DoF");
    std::vector<int32_t>().swap(owner);
    phase("hex order");

    // blocks: chunks of cells_per_block positions, halved while too many DoFs
    std::vector<uint64_t> keys(27 * (size_t)nc);
    const int n_chunks = (nc + cells_per_block - 1) / cells_per_block;
    std::vector<std::vector<std::pair<int, int>>> parts(n_chunks);
#pragma omp parallel for schedule(dynamic, 16)
    for (int k = 0; k < n_chunks; ++k)
        split_block(fs, cb.perm, k * cells_per_block, std::min(nc, (k + 1) * cells_per_block), max_dofs, keys.data(),
                    parts[k]);
    cb.cell_start.push_back(0);
    cb.dof_start.push_back(0);
    for (const auto& pv : parts)
        for (const auto& pd : pv) {
            cb.max_cells = std::max(cb.max_cells, pd.first - cb.cell_start.back());
            cb.max_dofs = std::max(cb.max_dofs, pd.second);
            cb.cell_start.push_back(pd.first);
            cb.dof_start.push_back(cb.dof_start.back() + pd.second);
        }
    cb.n_blocks = (int)cb.cell_start.size() - 1;
    phase("block cuts (sorted keys)");
    const int64_t ne = cb.dof_start.back();
    FGB_REQUIRE(ne < (int64_t)1 << 31, "too many block-local DoFs");
    cb.dof_list.resize(ne);
    cb.item_end.resize(ne);
    cb.slot.resize(ne);
    cb.loc.resize(27 * (size_t)nc);
    cb.items.assign(28 * (size_t)nc, 0);

    // local DoFs, items and completeness per block; slots numbered in block order
    std::vector<int32_t> n_inc(cb.n_blocks + 1, 0);
#pragma omp parallel for schedule(dynamic, 64)
    for (int b = 0; b < cb.n_blocks; ++b) {
        const int p0 = cb.cell_start[b], p1 = cb.cell_start[b + 1];
        const uint64_t* kb = keys.data() + 27 * (size_t)p0;
        const int m = 27 * (p1 - p0);
        int k = -1, inc = 0;
        for (int e = 0; e < m; ++e) {
            const int32_t dof = (int32_t)(kb[e] >> 16);
            const int item = (int)(kb[e] & 0xffff);
            if (e == 0 || dof != (int32_t)(kb[e - 1] >> 16)) {
                ++k;
                cb.dof_list[cb.dof_start[b] + k] = dof;
            }
            cb.items[28 * (size_t)p0 + e] = (uint16_t)item;
            cb.loc[27 * (size_t)p0 + item] = (uint16_t)k;
            cb.item_end[cb.dof_start[b] + k] = (uint16_t)(e + 1);
        }
        for (int q = cb.dof_start[b]; q < cb.dof_start[b + 1]; ++q) {
            const int dof = cb.dof_list[q];
            const int e0 = q == cb.dof_start[b] ? 0 : cb.item_end[q - 1];
            const bool complete = cb.item_end[q] - e0 == fs.r2c_ptr[dof + 1] - fs.r2c_ptr[dof];
            cb.slot[q] = complete ? -1 : inc++;
        }
        n_inc[b + 1] = inc;
    }
    std::vector<uint64_t>().swap(keys);
    phase("local DoFs, items");
    for (int b = 0; b < cb.n_blocks; ++b) n_inc[b + 1] += n_inc[b];
    cb.n_slots = n_inc[cb.n_blocks];
    std::vector<int32_t> slot_dof(cb.n_slots);
#pragma omp parallel for schedule(static)
    for (int b = 0; b < cb.n_blocks; ++b)
        for (int q = cb.dof_start[b]; q < cb.dof_start[b + 1]; ++q)
            if (cb.slot[q] >= 0) {
                cb.slot[q] += n_inc[b];
                slot_dof[cb.slot[q]] = cb.dof_list[q];
            }

    // slots renumbered by DoF: the slots of boundary DoF j are bnd_ptr[j] .. bnd_ptr[j+1]-1 in
    // ascending block order (block-order slot s ascends with the block). Counts per DoF, the
    // DoFs with slots compacted in ascending order (blocked scan), the slots bucketed by DoF
    // (atomic cursors) and each bucket sorted: the numbering of a sequential pass.
    std::vector<int32_t> cnt(n, 0);
#pragma omp parallel for schedule(static)
    for (int s = 0; s < cb.n_slots; ++s) __atomic_fetch_add(&cnt[slot_dof[s]], 1, __ATOMIC_RELAXED);
    std::vector<int32_t> first(n, -1);
    {
        const int nt = std::max(1, omp_get_max_threads());
        std::vector<int64_t> tn(nt + 1, 0), ts(nt + 1, 0);
        int n_bnd = 0;
#pragma omp parallel num_threads(nt)
        {
            const int t = omp_get_thread_num();
            const int d0 = (int)((int64_t)n * t / nt), d1 = (int)((int64_t)n * (t + 1) / nt);
            int64_t a = 0, b = 0;
            for (int d = d0; d < d1; ++d)
                if (cnt[d]) {
                    ++a;
                    b += cnt[d];
                }
            tn[t + 1] = a;
            ts[t + 1] = b;
#pragma omp barrier
#pragma omp single
            {
                for (int u = 0; u < nt; ++u) {
                    tn[u + 1] += tn[u];
                    ts[u + 1] += ts[u];
                }
                n_bnd = (int)tn[nt];
                cb.bnd_dofs.resize(n_bnd);
                cb.bnd_ptr.resize(n_bnd + 1);
                cb.bnd_ptr[n_bnd] = (int32_t)ts[nt];
            }
            int64_t j = tn[t], off = ts[t];
            for (int d = d0; d < d1; ++d)
                if (cnt[d]) {
                    cb.bnd_dofs[j] = d;
                    cb.bnd_ptr[j] = (int32_t)off;
                    first[d] = (int32_t)off;
                    off += cnt[d];
                    ++j;
                }
        }
        FGB_REQUIRE(cb.bnd_ptr[n_bnd] == cb.n_slots, "cell blocks: slot count");
    }
    std::vector<int32_t> order(cb.n_slots), renum(cb.n_slots);
    {
        std::vector<int32_t>& cur = first;  // bucket cursors from here on
#pragma omp parallel for schedule(static)
        for (int s = 0; s < cb.n_slots; ++s) order[__atomic_fetch_add(&cur[slot_dof[s]], 1, __ATOMIC_RELAXED)] = s;
        const int n_bnd = (int)cb.bnd_dofs.size();
#pragma omp parallel for schedule(dynamic, 4096)
        for (int j = 0; j < n_bnd; ++j) std::sort(order.begin() + cb.bnd_ptr[j], order.begin() + cb.bnd_ptr[j + 1]);
#pragma omp parallel for schedule(static)
        for (int p = 0; p < cb.n_slots; ++p) renum[order[p]] = p;
    }
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < ne; ++q)
        if (cb.slot[q] >= 0) cb.slot[q] = renum[cb.slot[q]];
    phase("slots");
    return cb;
}

namespace {
template <typename T>
void digest(uint64_t& h, const std::vector<T>& v) {
    const unsigned char* b = reinterpret_cast<const unsigned char*>(v.data());
    for (size_t i = 0; i < v.size() * sizeof(T); ++i) h = (h ^ b[i]) * 1099511628211ull;
}
}  // namespace

uint64_t validate_cell_blocks(const FemStructure& fs, const CellBlocks& cb, int cells_per_block, int max_dofs) {
    const int nc = fs.n_cells, n = fs.n_dofs;
    FGB_REQUIRE(cb.n_cells == nc && cb.n_dofs == n && (int)cb.perm.size() == nc, "cell blocks: sizes");
    std::vector<char> seen(nc, 0);
    for (int p = 0; p < nc; ++p) {
        const int c = cb.perm[p];
        FGB_REQUIRE(c >= 0 && c < nc && !seen[c], "cell blocks: perm is not a permutation");
        seen[c] = 1;
        if (p) FGB_REQUIRE(fs.cell_dofs[27 * (size_t)c + 13] > fs.cell_dofs[27 * (size_t)cb.perm[p - 1] + 13],
                           "cell blocks: cells not in interior-DoF order");
    }
    FGB_REQUIRE((int)cb.cell_start.size() == cb.n_blocks + 1 && cb.cell_start[0] == 0 && cb.cell_start.back() == nc,
                "cell blocks: block ranges");
    FGB_REQUIRE((int)cb.dof_start.size() == cb.n_blocks + 1 && cb.dof_start[0] == 0 &&
                    cb.dof_start.back() == (int64_t)cb.dof_list.size(),
                "cell blocks: local DoF ranges");
    std::vector<int32_t> total(n, 0), blocks_of(n, 0), complete_in(n, -1);
    for (int b = 0; b < cb.n_blocks; ++b) {
        const int p0 = cb.cell_start[b], nb = cb.cell_start[b + 1] - p0;
        const int q0 = cb.dof_start[b], nq = cb.dof_start[b + 1] - q0;
        FGB_REQUIRE(nb >= 1 && nb <= cells_per_block && nb <= cb.max_cells, "cell blocks: block size");
        FGB_REQUIRE(nq >= 1 && nq <= max_dofs && nq <= cb.max_dofs, "cell blocks: block DoF count");
        std::vector<char> used(27 * (size_t)nb, 0);
        for (int k = 0; k < nq; ++k) {
            const int dof = cb.dof_list[q0 + k];
            FGB_REQUIRE(dof >= 0 && dof < n, "cell blocks: DoF id");
            if (k) FGB_REQUIRE(dof > cb.dof_list[q0 + k - 1], "cell blocks: local DoFs not ascending");
            const int e0 = k ? cb.item_end[q0 + k - 1] : 0, e1 = cb.item_end[q0 + k];
            FGB_REQUIRE(e1 > e0 && e1 <= 27 * nb, "cell blocks: item range");
            for (int e = e0; e < e1; ++e) {
                const int it = cb.items[28 * (size_t)p0 + e];
                FGB_REQUIRE(it < 27 * nb && !used[it], "cell blocks: item repeated or out of range");
                if (e > e0) FGB_REQUIRE(it > cb.items[28 * (size_t)p0 + e - 1], "cell blocks: items not ascending");
                used[it] = 1;
                const int p = p0 + it / 27, l = it % 27;
                FGB_REQUIRE(fs.cell_dofs[27 * (size_t)cb.perm[p] + l] == dof, "cell blocks: item maps to another DoF");
                FGB_REQUIRE(cb.loc[27 * (size_t)p + l] == k, "cell blocks: loc does not map back");
            }
            const int cnt = e1 - e0, want = fs.r2c_ptr[dof + 1] - fs.r2c_ptr[dof];
            total[dof] += cnt;
            ++blocks_of[dof];
            if (cnt == want) {
                FGB_REQUIRE(cb.slot[q0 + k] == -1 && complete_in[dof] < 0, "cell blocks: complete DoF with a slot");
                complete_in[dof] = b;
            } else {
                FGB_REQUIRE(cb.slot[q0 + k] >= 0 && cb.slot[q0 + k] < cb.n_slots, "cell blocks: split DoF without a slot");
            }
        }
        for (int it = 0; it < 27 * nb; ++it) FGB_REQUIRE(used[it], "cell blocks: product not summed");
    }
    // split DoFs: one slot per block, ascending block = ascending slot, slots bnd_ptr[j].. of j
    FGB_REQUIRE((int)cb.bnd_ptr.size() == (int)cb.bnd_dofs.size() + 1 && cb.bnd_ptr.back() == cb.n_slots,
                "cell blocks: split-DoF ranges");
    std::vector<int32_t> bnd_index(n, -1);
    for (size_t j = 0; j < cb.bnd_dofs.size(); ++j) {
        const int d = cb.bnd_dofs[j];
        FGB_REQUIRE(bnd_index[d] < 0 && (j == 0 || d > cb.bnd_dofs[j - 1]), "cell blocks: split DoFs not ascending");
        bnd_index[d] = (int)j;
    }
    std::vector<int32_t> next_slot(cb.bnd_dofs.size(), 0);
    for (size_t j = 0; j < cb.bnd_dofs.size(); ++j) next_slot[j] = cb.bnd_ptr[j];
    for (int b = 0; b < cb.n_blocks; ++b)
        for (int q = cb.dof_start[b]; q < cb.dof_start[b + 1]; ++q) {
            if (cb.slot[q] < 0) continue;
            const int j = bnd_index[cb.dof_list[q]];
            FGB_REQUIRE(j >= 0 && cb.slot[q] == next_slot[j]++, "cell blocks: slots not in block order");
        }
    for (int d = 0; d < n; ++d) {
        const int want = fs.r2c_ptr[d + 1] - fs.r2c_ptr[d];
        FGB_REQUIRE(total[d] == want, "cell blocks: DoF products do not cover its cells");
        const bool split = bnd_index[d] >= 0;
        FGB_REQUIRE(split != (complete_in[d] >= 0), "cell blocks: DoF neither complete nor split");
        if (split) FGB_REQUIRE(cb.bnd_ptr[bnd_index[d] + 1] - cb.bnd_ptr[bnd_index[d]] == blocks_of[d] &&
                                   next_slot[bnd_index[d]] == cb.bnd_ptr[bnd_index[d] + 1],
                               "cell blocks: split DoF slot count");
    }
    uint64_t h = 1469598103934665603ull;
    digest(h, cb.perm); digest(h, cb.cell_start); digest(h, cb.dof_start); digest(h, cb.dof_list);
    digest(h, cb.item_end); digest(h, cb.slot); digest(h, cb.loc); digest(h, cb.items);
    digest(h, cb.bnd_dofs); digest(h, cb.bnd_ptr);
    return h;
}

}  // namespace fgb
