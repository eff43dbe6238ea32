// Host-side mesh plan: locality reordering, tiles and per-tetra reference quantities.
//
// The reference keeps the user's node and tetra order and recomputes the inverse reference
// edge matrix every step (tetra.cl:47-53). Here, once at set-up:
//  * nodes are sorted along a Morton (Z-order) curve of their reference positions, and tetrahedra
//    along the Morton curve of their centroids, so a run of consecutive tetrahedra touches a
//    compact set of nodes;
//  * tetrahedra are grouped into tiles of at most tile_tets (128, 256 or 512) elements and
//    min(tile_tets, 256) distinct nodes by greedy region growing: a tile starts at the first
//    unassigned tetra along the Morton curve and repeatedly takes the adjacent tetra that adds
//    the fewest new nodes, so tiles are compact and share few nodes (every node entry of a tile
//    costs a displacement gather and three accumulator atomics per step). Each tetra's corners
//    are stored as 8-bit indices into its tile's node list, plus the tile's incidence list
//    (corners grouped by node) for the fixed-order force sums;
//  * Dm^-1 (inverse of the reference edge matrix [X1-X0, X2-X0, X3-X0]) and the signed
//    reference volume V0 = det(Dm)/6 (TetraCell.py:33-41) are computed in double and stored
//    as float;
//  * reference positions are split into float hi + lo parts.
// Corner order within a tetra is the user's, so node 0 of each tetra stays the base node of
// the reference's elastic kernel (tetra.cl:31-35).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

#include "nfx_internal.h"

namespace nfx {

namespace {

inline uint64_t spread3(uint64_t x) {
    x &= 0x1fffff;  // 21 bits
    x = (x | (x << 32)) & 0x1f00000000ffffULL;
    x = (x | (x << 16)) & 0x1f0000ff0000ffULL;
    x = (x | (x << 8)) & 0x100f00f00f00f00fULL;
    x = (x | (x << 4)) & 0x10c30c30c30c30c3ULL;
    x = (x | (x << 2)) & 0x1249249249249249ULL;
    return x;
}

inline uint64_t morton3(uint64_t x, uint64_t y, uint64_t z) { return spread3(x) | (spread3(y) << 1) | (spread3(z) << 2); }

struct Quant {
    double lo[3];
    double inv_h;
    uint64_t q(double v, int d) const {
        double s = (v - lo[d]) * inv_h;
        if (!(s > 0)) s = 0;
        if (s > 2097151.0) s = 2097151.0;
        return (uint64_t)s;
    }
};

// Greedy region-growing tiles (see the file comment). seed_order: the tetrahedra in Morton
// order. Appends each tile's tetrahedra to tets and the tiles' end offsets to tile_end.
// Candidates are kept in five FIFO buckets by the number of nodes they would add (0..4); a
// bucket entry is stale when the tetra was assigned or its count dropped since it was pushed.
void grow_tiles(int64_t np, int64_t nt, const uint32_t* T, const std::vector<int64_t>& seed_order, int tile_tets,
                int nodes_max, std::vector<uint32_t>& tets, std::vector<int64_t>& tile_end) {
    std::vector<int64_t> off((size_t)np + 1, 0);  // node -> incident tetrahedra (CSR)
    for (int64_t i = 0; i < 4 * nt; i++) off[(size_t)T[i] + 1]++;
    for (int64_t i = 0; i < np; i++) off[i + 1] += off[i];
    std::vector<uint32_t> adj((size_t)(4 * nt));
    {
        std::vector<int64_t> fill(off.begin(), off.end() - 1);
        for (int64_t k = 0; k < 4; k++)
            for (int64_t t = 0; t < nt; t++) adj[fill[T[k * nt + t]]++] = (uint32_t)t;
    }
    std::vector<uint8_t> assigned((size_t)nt, 0), newc((size_t)nt, 0);
    std::vector<int64_t> node_stamp((size_t)np, -1), tet_stamp((size_t)nt, -1);
    std::vector<uint32_t> bucket[5];
    size_t head[5];
    tets.clear();
    tets.reserve((size_t)nt);
    tile_end.clear();
    int64_t seed = 0, tile = 0;
    for (;;) {
        while (seed < nt && assigned[seed_order[seed]]) seed++;
        if (seed == nt) break;
        for (int b = 0; b < 5; b++) {
            bucket[b].clear();
            head[b] = 0;
        }
        int nodes = 0, cnt = 0;
        auto new_nodes = [&](uint32_t t) {
            int c = 0;
            for (int k = 0; k < 4; k++) c += node_stamp[T[k * nt + t]] != tile;
            return c;
        };
        auto add = [&](uint32_t t) {
            assigned[t] = 1;
            tets.push_back(t);
            cnt++;
            for (int k = 0; k < 4; k++) {
                const uint32_t n = T[k * nt + t];
                if (node_stamp[n] == tile) continue;
                node_stamp[n] = tile;
                nodes++;
                for (int64_t a = off[n]; a < off[n + 1]; a++) {
                    const uint32_t t2 = adj[a];
                    if (assigned[t2]) continue;
                    if (tet_stamp[t2] != tile) {
                        tet_stamp[t2] = tile;
                        newc[t2] = (uint8_t)new_nodes(t2);
                    } else if (newc[t2] > 0) {
                        newc[t2]--;
                    }
                    bucket[newc[t2]].push_back(t2);
                }
            }
        };
        add((uint32_t)seed_order[seed]);
        while (cnt < tile_tets) {
            int64_t pick = -1;
            for (int b = 0; b < 5 && pick < 0; b++) {
                if (nodes + b > nodes_max) break;
                while (head[b] < bucket[b].size()) {
                    const uint32_t t = bucket[b][head[b]++];
                    if (!assigned[t] && tet_stamp[t] == tile && newc[t] == b) {
                        pick = t;
                        break;
                    }
                }
            }
            if (pick < 0) {  // nothing adjacent fits: the next unassigned tetra along the curve
                while (seed < nt && assigned[seed_order[seed]]) seed++;
                if (seed == nt) break;
                const uint32_t t = (uint32_t)seed_order[seed];
                if (nodes + new_nodes(t) > nodes_max) break;
                pick = t;
            }
            add((uint32_t)pick);
        }
        tile_end.push_back((int64_t)tets.size());
        tile++;
    }
}

}  // namespace

bool build_mesh_plan(int64_t np, int64_t nt, const double* P, const uint32_t* T, int tile_tets, MeshPlan& plan,
                     std::string& err) {
    if (tile_tets != 64 && tile_tets != 128 && tile_tets != 256 && tile_tets != 512) {
        err = "tile size must be 64, 128, 256 or 512";
        return false;
    }
    if (np <= 0 || nt <= 0) {
        err = "mesh needs at least one node and one tetra";
        return false;
    }
    if (np > (int64_t)0x7fffffff || nt > (int64_t)0x7fffffff) {
        err = "mesh too large (more than 2^31-1 nodes or tetrahedra)";
        return false;
    }
    for (int64_t t = 0; t < 4 * nt; t++) {
        if ((int64_t)T[t] >= np) {
            err = "tetra corner index out of range";
            return false;
        }
    }
    for (int64_t i = 0; i < 3 * np; i++) {
        if (!std::isfinite(P[i])) {
            err = "non-finite node position";
            return false;
        }
    }
    plan = MeshPlan();
    plan.np = np;
    plan.nt = nt;
    plan.tile_tets = tile_tets;
    const int64_t nodes_max = std::min<int64_t>(TILE_NODES_MAX, tile_tets);

    // quantisation: cell size ~ mean node spacing
    Quant Q;
    double hi[3];
    for (int d = 0; d < 3; d++) {
        Q.lo[d] = P[d * np];
        hi[d] = P[d * np];
        for (int64_t i = 1; i < np; i++) {
            Q.lo[d] = std::min(Q.lo[d], P[d * np + i]);
            hi[d] = std::max(hi[d], P[d * np + i]);
        }
    }
    double vol = 1.0;
    for (int d = 0; d < 3; d++) vol *= std::max(hi[d] - Q.lo[d], 1e-12);
    double h = std::cbrt(vol / (double)np);
    if (!(h > 0)) h = 1.0;
    Q.inv_h = 1.0 / h;

    // nodes
    std::vector<uint64_t> nkey(np);
    for (int64_t i = 0; i < np; i++)
        nkey[i] = morton3(Q.q(P[i], 0), Q.q(P[np + i], 1), Q.q(P[2 * np + i], 2));
    plan.node_user.resize(np);
    std::iota(plan.node_user.begin(), plan.node_user.end(), 0);
    std::stable_sort(plan.node_user.begin(), plan.node_user.end(),
                     [&](int64_t a, int64_t b) { return nkey[a] < nkey[b]; });
    plan.node_int.resize(np);
    for (int64_t i = 0; i < np; i++) plan.node_int[plan.node_user[i]] = i;

    // tetrahedra, by centroid
    std::vector<uint64_t> tkey(nt);
    for (int64_t t = 0; t < nt; t++) {
        double c[3] = {0, 0, 0};
        for (int k = 0; k < 4; k++) {
            const int64_t n = T[k * nt + t];
            for (int d = 0; d < 3; d++) c[d] += 0.25 * P[d * np + n];
        }
        tkey[t] = morton3(Q.q(c[0], 0), Q.q(c[1], 1), Q.q(c[2], 2));
    }
    std::vector<int64_t> order(nt);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return tkey[a] < tkey[b]; });

    // Tiles at a fixed stride: tile b owns tetra slots [b*T, b*T + T) and node-list entries
    // [b*NMAX, b*NMAX + NMAX); unused slots and entries are zero padding (a padding tetra has
    // Dm^-1 = 0 and V0 = 0 and produces no force; a padding node entry has count 0). Kernels can
    // then address a tile's data without first loading its offsets.
    const int64_t T_ = tile_tets, NM_ = nodes_max;
    std::vector<uint32_t> tile_tets_list;
    std::vector<int64_t> tile_end;
    grow_tiles(np, nt, T, order, tile_tets, (int)nodes_max, tile_tets_list, tile_end);
    order.assign(tile_tets_list.begin(), tile_tets_list.end());  // tetrahedra in tile order
    std::vector<int64_t> slot_user;  // tetra slot -> user tetra (-1: padding)
    std::vector<uint32_t> ids;
    ids.reserve(4 * (size_t)tile_tets);
    int64_t t0 = 0, b = 0;
    while (t0 < nt) {
        const int64_t cnt = tile_end[b] - t0;
        ids.clear();
        for (int64_t j = 0; j < cnt; j++) {
            const int64_t ut = order[t0 + j];
            for (int k = 0; k < 4; k++) ids.push_back((uint32_t)plan.node_int[T[k * nt + ut]]);
        }
        std::sort(ids.begin(), ids.end());
        ids.erase(std::unique(ids.begin(), ids.end()), ids.end());
        const size_t nn = ids.size();
        const size_t s0 = (size_t)(b * T_);
        slot_user.resize(s0 + T_, -1);
        plan.lconn.resize(4 * (s0 + T_), 0);
        plan.tile_inc.resize(4 * (s0 + T_), 0);
        // Local node order: by incidence count, largest first (ties by node index). The thread of
        // local node q sums its corners in a loop, and a warp runs as many iterations as its
        // largest count, so grouping similar counts into the same warp saves iterations.
        std::vector<uint32_t> cnt_by_id(nn, 0);
        for (int64_t j = 0; j < cnt; j++) {
            const int64_t ut = order[t0 + j];
            for (int k = 0; k < 4; k++) {
                const uint32_t g = (uint32_t)plan.node_int[T[k * nt + ut]];
                cnt_by_id[std::lower_bound(ids.begin(), ids.end(), g) - ids.begin()]++;
            }
        }
        std::vector<uint32_t> by_count(nn), loc_of(nn);
        std::iota(by_count.begin(), by_count.end(), 0u);
        std::stable_sort(by_count.begin(), by_count.end(),
                         [&](uint32_t a, uint32_t c) { return cnt_by_id[a] > cnt_by_id[c]; });
        for (size_t q = 0; q < nn; q++) loc_of[by_count[q]] = (uint32_t)q;
        std::vector<uint32_t> count(nn, 0), first(nn, 0);
        for (int64_t j = 0; j < cnt; j++) {
            const int64_t ut = order[t0 + j];
            slot_user[s0 + j] = ut;
            for (int k = 0; k < 4; k++) {
                const uint32_t g = (uint32_t)plan.node_int[T[k * nt + ut]];
                const uint32_t loc = loc_of[std::lower_bound(ids.begin(), ids.end(), g) - ids.begin()];
                plan.lconn[4 * (s0 + j) + k] = (uint8_t)loc;
                count[loc]++;
            }
        }
        // incidence list of the tile: corners grouped by local node, in (tet, corner) order, each
        // entry the corner's slot in the kernels' corner-major shared array (corner * T + tet)
        for (size_t q = 1; q < nn; q++) first[q] = first[q - 1] + count[q - 1];
        std::vector<uint32_t> fill(first);
        for (int64_t j = 0; j < cnt; j++)
            for (int k = 0; k < 4; k++) {
                const uint8_t loc = plan.lconn[4 * (s0 + j) + k];
                plan.tile_inc[4 * s0 + fill[loc]++] = (uint16_t)(k * T_ + j);
            }
        plan.tile_nodes.resize(2 * (size_t)((b + 1) * NM_), 0u);
        for (size_t q = 0; q < nn; q++) {
            plan.tile_nodes[2 * (b * NM_ + q)] = ids[by_count[q]];
            plan.tile_nodes[2 * (b * NM_ + q) + 1] = (first[q] << 16) | count[q];
        }
        plan.tile_meta.push_back((uint32_t)cnt | ((uint32_t)nn << 16));
        t0 += cnt;
        b++;
    }
    plan.ntiles = b;
    plan.nslots = b * T_;
    {
        // the most tiles any node appears in sets the per-tile bound of the fixed-point sums
        std::vector<int32_t> tiles_of((size_t)np, 0);
        for (int64_t q = 0; q < b; q++) {
            const int64_t nn = plan.tile_meta[q] >> 16;
            for (int64_t e = 0; e < nn; e++) tiles_of[plan.tile_nodes[2 * (q * NM_ + e)]]++;
        }
        plan.max_tiles_per_node = std::max(1, *std::max_element(tiles_of.begin(), tiles_of.end()));
        plan.fix_max = force_fix_bound(plan.max_tiles_per_node);
    }
    plan.tet_user = std::move(slot_user);
    plan.tile_tet_begin.resize(b + 1);
    plan.tile_node_begin.resize(b + 1);
    for (int64_t q = 0; q <= b; q++) {
        plan.tile_tet_begin[q] = (int32_t)(q * T_);
        plan.tile_node_begin[q] = (int32_t)(q * NM_);
    }

    // per-tetra Dm^-1 and V0 (slot order; padding slots stay zero), and the lumped nodal masses of
    // density 1 that VelocityVerlet2 uses: a quarter of every tetra's V0 to each of its corners
    // (SimulationLegacy.py:911-924)
    plan.dmi.assign(12 * (size_t)plan.nslots, 0.0f);
    std::vector<double> mass((size_t)np, 0.0);
    for (int64_t it = 0; it < plan.nslots; it++) {
        const int64_t ut = plan.tet_user[it];
        if (ut < 0) continue;
        const int64_t n0 = T[ut];
        double M[9];  // columns X_k - X_0
        for (int k = 0; k < 3; k++) {
            const int64_t nk = T[(k + 1) * nt + ut];
            for (int d = 0; d < 3; d++) M[3 * d + k] = P[d * np + nk] - P[d * np + n0];
        }
        const double A[9] = {M[4] * M[8] - M[5] * M[7], M[2] * M[7] - M[1] * M[8], M[1] * M[5] - M[2] * M[4],
                             M[5] * M[6] - M[3] * M[8], M[0] * M[8] - M[2] * M[6], M[2] * M[3] - M[0] * M[5],
                             M[3] * M[7] - M[4] * M[6], M[1] * M[6] - M[0] * M[7], M[0] * M[4] - M[1] * M[3]};
        const double det = M[0] * A[0] + M[1] * A[3] + M[2] * A[6];
        if (det == 0.0 || !std::isfinite(det)) {
            err = "degenerate tetra (zero reference volume) at index " + std::to_string(ut);
            return false;
        }
        float* o = &plan.dmi[12 * it];
        for (int k = 0; k < 9; k++) o[k] = (float)(A[k] / det);
        o[9] = (float)(det / 6.0);
        for (int k = 0; k < 4; k++) mass[T[k * nt + ut]] += 0.25 * (det / 6.0);
    }

    // reference positions, hi/lo, internal order
    plan.Xh.assign(4 * (size_t)np, 0.0f);
    plan.Xl.assign(4 * (size_t)np, 0.0f);
    for (int64_t i = 0; i < np; i++) {
        const int64_t u = plan.node_user[i];
        for (int d = 0; d < 3; d++) {
            const double x = P[d * np + u];
            const float h32 = (float)x;
            plan.Xh[4 * i + d] = h32;
            plan.Xl[4 * i + d] = (float)(x - (double)h32);
        }
        // the unused fourth lane carries the inverse lumped mass (density 1); 0 for a node no
        // tetra touches
        const double m = mass[u];
        plan.Xh[4 * i + 3] = m != 0.0 ? (float)(1.0 / m) : 0.0f;
    }

    // bounding box of every node block's reference positions, rounded outwards to float
    const int64_t nb = (np + NODE_BLOCK - 1) / NODE_BLOCK;
    plan.block_box.assign(8 * (size_t)nb, 0.0f);
    for (int64_t q = 0; q < nb; q++) {
        double lo[3] = {HUGE_VAL, HUGE_VAL, HUGE_VAL}, hi[3] = {-HUGE_VAL, -HUGE_VAL, -HUGE_VAL};
        for (int64_t i = q * NODE_BLOCK; i < std::min<int64_t>(np, (q + 1) * NODE_BLOCK); i++) {
            const int64_t u = plan.node_user[i];
            for (int d = 0; d < 3; d++) {
                lo[d] = std::min(lo[d], P[d * np + u]);
                hi[d] = std::max(hi[d], P[d * np + u]);
            }
        }
        for (int d = 0; d < 3; d++) {
            float l = (float)lo[d], h = (float)hi[d];
            if ((double)l > lo[d]) l = std::nextafter(l, -HUGE_VALF);
            if ((double)h < hi[d]) h = std::nextafter(h, HUGE_VALF);
            plan.block_box[8 * q + d] = l;
            plan.block_box[8 * q + 4 + d] = h;
        }
    }
    return true;
}

}  // namespace nfx
