// Batched cells (C ABI nfx_batch_*): many independent cells of uneven size and material advance
// together. Each cell's mesh gets its own plan (reordering, tiles, Dm^-1), built on host threads.
// Cells are grouped by size into buckets (small, medium, large), and every bucket has its own tile
// size — chosen per bucket by the autotuner, which times each candidate on a sample of that
// bucket's cells. The node state of all cells is one set of arrays (every cell's nodes occupy
// whole node blocks, so the node pass maps a block to one cell); each bucket has its own tile and
// per-tetra arrays (every tile belongs to one cell, so the element pass maps a tile to one cell).
// One element-pass launch per bucket and one node-pass launch advance all cells per step, and
// chunks of steps are captured as a CUDA graph. The reference has no batched mode: its equivalent
// is one Simulation per cell (nofluidx3d/Simulation.py:35).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <map>
#include <memory>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/nfx.h"
#include "nfx_internal.h"

using namespace nfx;

namespace {

constexpr int BATCH_GRAPH_STEPS = 50;

int bfail(int code, const std::string& msg) {
    set_error(msg);
    return code;
}

#define BCUDA(expr)                                                                                         \
    do {                                                                                                    \
        cudaError_t e_ = (expr);                                                                            \
        if (e_ != cudaSuccess) return bfail(NFX_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define BARG(cond, msg)                              \
    do {                                             \
        if (!(cond)) return bfail(NFX_ERR_ARG, msg); \
    } while (0)

struct CellHost {
    int64_t np = 0, nt = 0;
    std::vector<double> points;   // 3*np SoA (empty when the mesh is another cell's)
    std::vector<uint32_t> tets;   // 4*nt SoA
    int mesh_src = -1;            // cell whose mesh this cell shares, -1: its own
    MaterialDev mat{};
    bool has_mat = false;
    int n_contacts = 0;
    ContactDev c[MAX_CONTACTS]{};
    double xi = 0.005;
    bool fix_top_bottom = false;
    int integrator = INTEGRATOR_VV;
    double density = 1.0;
    int si_contact = -1;
    std::shared_ptr<MeshPlan> plan;  // shared by every cell with the same mesh
    // placement in the concatenated arrays
    int64_t node_base = 0, tet_base = 0, tile_base = 0, block_base = 0, nblocks = 0;
};

// Size classes of the buckets, by tetra count: small cells (up to 32,768 tetra), medium (up to
// 262,144) and large. Cells that share a mesh have the same count and so the same bucket.
constexpr int MAX_BUCKETS = 3;
inline int size_class(int64_t nt) { return nt <= 32768 ? 0 : (nt <= 262144 ? 1 : 2); }

// One bucket's element-pass view: its own tile arrays and per-tetra state, the batch's node
// arrays and cell table. mesh.np is the whole batch's node count (the accumulator's stride) and
// mesh.tile_base the bucket's first tile in the batch-wide tile numbering.
struct BucketDev {
    int tile_tets = DEFAULT_TILE_TETS;
    int64_t cells = 0, tets = 0;
    MeshDev mesh{};
    StateDev st{};
    BatchDev bd{};
};

// Device arrays of one built batch (a full batch, or a sub-batch the autotuner times).
struct BatchDevice {
    std::vector<void*> allocs;
    MeshDev mesh{};  // node-pass view: node arrays of every cell, all tiles counted
    StateDev st{};   // node state and control words (per-tetra arrays live in the buckets)
    BatchDev bd{};
    std::vector<BucketDev> buckets;
    int nblocks = 0;
    StepClock* d_clock = nullptr;
    unsigned* d_status = nullptr;
    cudaGraphExec_t graph = nullptr;
    void release() {
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
        for (void* p : allocs) cudaFree(p);
        allocs.clear();
    }
};

}  // namespace

struct nfx_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    int tile_tets = 0;  // 0: chosen by the autotuner at finalize
    int model = -1;
    std::vector<CellHost> cells;
    bool finalized = false;
    int record_contact = -1;
    long long record_every = 0, max_rows = 0;
    BatchDevice dev;
    long long time = 0;
    long long rows_written = 0;
    std::vector<int> tuned;    // tile sizes the autotuner tried (per bucket, in bucket order)
    std::vector<float> tuned_ms;
    std::vector<int> tuned_bucket;
    long long* d_zero_meta = nullptr;
    bool has_si = false;  // some cell has an integrated sphere contact
};

namespace {

template <class T>
int balloc(std::vector<void*>& owner, T** p, size_t count) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
    if (e != cudaSuccess) return bfail(NFX_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    owner.push_back(q);
    *p = (T*)q;
    return NFX_OK;
}

int mesh_owner(const nfx_batch* b, int cell) {
    const int s = b->cells[cell].mesh_src;
    return s < 0 ? cell : s;
}

// Build the plans of the given cells with the given tile size on host threads: one plan per
// distinct mesh, shared by every cell that uses it.
int build_plans(nfx_batch* b, const std::vector<int>& which, int tile_tets) {
    std::vector<int> owners;
    for (int k : which) owners.push_back(mesh_owner(b, k));
    std::sort(owners.begin(), owners.end());
    owners.erase(std::unique(owners.begin(), owners.end()), owners.end());
    std::vector<std::shared_ptr<MeshPlan>> plans(owners.size());
    std::vector<std::string> errs(owners.size());
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    std::vector<std::thread> pool;
    std::atomic<size_t> next{0};
    auto work = [&]() {
        for (;;) {
            const size_t k = next.fetch_add(1);
            if (k >= owners.size()) return;
            const CellHost& c = b->cells[owners[k]];
            plans[k] = std::make_shared<MeshPlan>();
            if (!build_mesh_plan(c.np, c.nt, c.points.data(), c.tets.data(), tile_tets, *plans[k], errs[k]))
                errs[k] = "cell " + std::to_string(owners[k]) + ": " + errs[k];
        }
    };
    for (unsigned t = 0; t < std::min<size_t>(hw, owners.size()); t++) pool.emplace_back(work);
    for (auto& t : pool) t.join();
    for (auto& e : errs)
        if (!e.empty()) return bfail(NFX_ERR_ARG, e);
    for (int k : which) {
        const size_t o = std::lower_bound(owners.begin(), owners.end(), mesh_owner(b, k)) - owners.begin();
        b->cells[k].plan = plans[o];
    }
    return NFX_OK;
}

// Concatenate the plans of `which` into device arrays (zeroed state). bucket[k] is the bucket of
// cell which[k] and tiles[g] the tile size of bucket g; the cells' plans must have been built
// with their bucket's tile size. Cell index k of the device table is the position in `which`.
int build_device(nfx_batch* b, const std::vector<int>& which, const std::vector<int>& bucket,
                 const std::vector<int>& tiles, BatchDevice& D) {
    D.release();
    const int nbk = (int)tiles.size();
    int64_t np = 0, nblocks = 0;
    std::vector<int64_t> bk_tiles(nbk, 0), bk_slots(nbk, 0), bk_ntn(nbk, 0), bk_cells(nbk, 0), bk_tets(nbk, 0);
    for (size_t k = 0; k < which.size(); k++) {
        CellHost& c = b->cells[which[k]];
        const int g = bucket[k];
        if (c.plan->tile_tets != tiles[g]) return bfail(NFX_ERR_STATE, "internal: plan tile size differs from its bucket's");
        c.node_base = np;
        c.block_base = nblocks;
        c.nblocks = (c.np + NODE_BLOCK - 1) / NODE_BLOCK;
        np += c.nblocks * NODE_BLOCK;  // whole blocks per cell
        nblocks += c.nblocks;
        c.tet_base = bk_slots[g];   // within the bucket
        c.tile_base = bk_tiles[g];  // within the bucket (made batch-wide below)
        bk_slots[g] += c.plan->nslots;
        bk_tiles[g] += c.plan->ntiles;
        bk_ntn[g] += (int64_t)c.plan->tile_nodes.size() / 2;
        bk_cells[g]++;
        bk_tets[g] += c.nt;
    }
    std::vector<int64_t> bk_tile_base(nbk, 0);
    int64_t ntiles = 0;
    for (int g = 0; g < nbk; g++) {
        bk_tile_base[g] = ntiles;
        ntiles += bk_tiles[g];
        if (bk_slots[g] > 0x7fffffff) return bfail(NFX_ERR_ARG, "batch too large");
    }
    if (np > 0x7fffffff) return bfail(NFX_ERR_ARG, "batch too large");
    auto& A = D.allocs;
    int rc;
    cudaStream_t st = b->stream;
    const size_t rows = (size_t)std::max<long long>(b->max_rows, 1);

    // node arrays and the cell table
    std::vector<float> Xh(4 * (size_t)np, 0.f), Xl(4 * (size_t)np, 0.f), box(8 * (size_t)nblocks, 0.f);
    std::vector<int> block_cell(nblocks);
    std::vector<CellDev> cells(which.size());
    float fix_max = FORCE_FIX_MAX;
    for (size_t k = 0; k < which.size(); k++) {
        CellHost& c = b->cells[which[k]];
        const MeshPlan& P = *c.plan;
        std::memcpy(&Xh[4 * c.node_base], P.Xh.data(), P.Xh.size() * sizeof(float));
        std::memcpy(&Xl[4 * c.node_base], P.Xl.data(), P.Xl.size() * sizeof(float));
        for (int64_t q = 0; q < c.nblocks; q++) block_cell[c.block_base + q] = (int)k;
        std::memcpy(&box[8 * c.block_base], P.block_box.data(), P.block_box.size() * sizeof(float));
        fix_max = std::min(fix_max, P.fix_max);
        CellDev& C = cells[k];
        C.mat = c.mat;
        C.n_contacts = c.n_contacts;
        for (int q = 0; q < c.n_contacts; q++) {
            C.c[q] = c.c[q];
            C.c[q].table = nullptr;
            C.c[q].meta = b->d_zero_meta;
        }
        const double xi = c.xi;
        C.vv_a = (float)((1 - 0.5 * xi) / (1 + 0.5 * xi));
        C.vv_hb = (float)(0.5 / (1 + 0.5 * xi));
        C.vv_dm = (float)(1 - 0.5 * xi);
        C.integrator = c.integrator;
        C.vv2_c = (float)(1.0 / (1.0 + 0.5 * xi));
        C.vv2_xi = (float)xi;
        C.inv_density = (float)(1.0 / c.density);
        C.si_contact = c.si_contact;
        C.tile_begin = (int)(bk_tile_base[bucket[k]] + c.tile_base);
        C.tile_end = (int)(C.tile_begin + P.ntiles);
        C.fix_a = C.fix_b = -1;
        if (c.fix_top_bottom && c.integrator == INTEGRATOR_VV) {
            if (c.np > 3) C.fix_a = (int)(c.node_base + P.node_int[3]);
            if (c.np > 4) C.fix_b = (int)(c.node_base + P.node_int[4]);
        }
        C.record_contact = b->record_contact < c.n_contacts ? b->record_contact : -1;
        C.node_begin = (int)c.node_base;
        C.node_end = (int)(c.node_base + c.np);
        C.block_begin = (int)c.block_base;
        C.block_end = (int)(c.block_base + c.nblocks);
    }
    float4 *d_xh, *d_xl, *d_ua, *d_va; float2 *d_ub, *d_vb; unsigned long long* d_fa; double* d_part; double* d_fout;
    double* d_tpart; CellDev* d_cells; int* d_bc; unsigned* d_cc; unsigned* d_cst; double* d_curves = nullptr;
    float4* d_box;
    if ((rc = balloc(A, &d_xh, np)) || (rc = balloc(A, &d_xl, np)) || (rc = balloc(A, &d_ua, np)) ||
        (rc = balloc(A, &d_ub, np)) || (rc = balloc(A, &d_va, np)) || (rc = balloc(A, &d_vb, np)) ||
        (rc = balloc(A, &d_fa, 3 * (size_t)np)) || (rc = balloc(A, &d_part, nblocks)) || (rc = balloc(A, &d_fout, cells.size())) ||
        (rc = balloc(A, &d_tpart, ntiles)) || (rc = balloc(A, &d_cells, cells.size())) || (rc = balloc(A, &d_bc, nblocks)) ||
        (rc = balloc(A, &d_cc, cells.size())) || (rc = balloc(A, &d_cst, cells.size())) ||
        (rc = balloc(A, &d_curves, 3 * rows * cells.size())) || (rc = balloc(A, &D.d_clock, 1)) ||
        (rc = balloc(A, &D.d_status, 1)) || (rc = balloc(A, &d_box, 2 * (size_t)nblocks)))
        return rc;
    BCUDA(cudaMemcpyAsync(d_box, box.data(), box.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    BCUDA(cudaMemcpyAsync(d_xh, Xh.data(), Xh.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    BCUDA(cudaMemcpyAsync(d_xl, Xl.data(), Xl.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    for (float4* z : {d_ua, d_va}) BCUDA(cudaMemsetAsync(z, 0, (size_t)np * sizeof(float4), st));
    for (float2* z : {d_ub, d_vb}) BCUDA(cudaMemsetAsync(z, 0, (size_t)np * sizeof(float2), st));
    BCUDA(cudaMemsetAsync(d_fa, 0, 3 * (size_t)np * sizeof(unsigned long long), st));
    BCUDA(cudaMemcpyAsync(d_cells, cells.data(), cells.size() * sizeof(CellDev), cudaMemcpyHostToDevice, st));
    BCUDA(cudaMemcpyAsync(d_bc, block_cell.data(), block_cell.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    BCUDA(cudaMemsetAsync(d_cc, 0, cells.size() * sizeof(unsigned), st));
    BCUDA(cudaMemsetAsync(d_cst, 0, cells.size() * sizeof(unsigned), st));
    BCUDA(cudaMemsetAsync(d_curves, 0, 3 * rows * cells.size() * sizeof(double), st));
    BCUDA(cudaMemsetAsync(D.d_clock, 0, sizeof(StepClock), st));
    BCUDA(cudaMemsetAsync(D.d_status, 0, sizeof(unsigned), st));
    BCUDA(cudaStreamSynchronize(st));  // the host vectors go out of scope
    MeshDev& M = D.mesh;
    M = MeshDev{};
    M.np = (int)np;
    M.ntiles = (int)ntiles;
    M.tile_tets = tiles.empty() ? DEFAULT_TILE_TETS : tiles[0];
    M.Xh = d_xh;
    M.Xl = d_xl;
    M.block_box = d_box;
    // cells share no nodes, so each cell's own bound keeps its words in range; the kernels take
    // one bound for the whole batch: the smallest
    M.fix_max = fix_max;
    StateDev& S = D.st;
    S = StateDev{};
    S.ua = d_ua;
    S.ub = d_ub;
    S.va = d_va;
    S.vb = d_vb;
    S.facc = d_fa;
    S.status = D.d_status;
    S.clock = D.d_clock;
    S.partials = d_part;
    S.tile_partials = d_tpart;
    S.force_out = d_fout;
    BatchDev& B = D.bd;
    B = BatchDev{};
    B.cells = d_cells;
    B.block_cell = d_bc;
    B.cell_counter = d_cc;
    B.cell_status = d_cst;
    B.curves = d_curves;
    B.record_every = b->record_contact >= 0 ? b->record_every : 0;
    B.max_rows = b->max_rows;
    B.fields_every = b->record_every;
    D.nblocks = (int)nblocks;

    // per bucket: tile arrays, per-tetra state, tile -> cell map
    D.buckets.assign(nbk, BucketDev{});
    for (int g = 0; g < nbk; g++) {
        BucketDev& K = D.buckets[g];
        K.tile_tets = tiles[g];
        K.cells = bk_cells[g];
        K.tets = bk_tets[g];
        const int64_t nt = bk_slots[g], nti = bk_tiles[g], ntn = bk_ntn[g];
        const size_t ntp = (size_t)nt + ARRAY_PAD;
        std::vector<int> tile_tet_begin(nti + 1), tile_node_begin(nti + 1), tile_cell(std::max<int64_t>(nti, 1));
        std::vector<unsigned> tile_meta(std::max<int64_t>(nti, 1));
        std::vector<uint32_t> tile_nodes(2 * (size_t)ntn);
        std::vector<uint8_t> lconn(4 * ntp, 0);
        std::vector<uint16_t> tile_inc(4 * ntp, 0);
        std::vector<float> da(4 * ntp, 0.f), db(4 * ntp, 0.f), dc(2 * ntp, 0.f);
        int64_t tn_pos = 0;
        for (size_t k = 0; k < which.size(); k++) {
            if (bucket[k] != g) continue;
            const CellHost& c = b->cells[which[k]];
            const MeshPlan& P = *c.plan;
            for (int64_t t = 0; t < P.ntiles; t++) {
                tile_tet_begin[c.tile_base + t] = (int)(c.tet_base + P.tile_tet_begin[t]);
                tile_node_begin[c.tile_base + t] = (int)(tn_pos + P.tile_node_begin[t]);
                tile_meta[c.tile_base + t] = P.tile_meta[t];
                tile_cell[c.tile_base + t] = (int)k;
            }
            for (size_t q = 0; q < P.tile_nodes.size() / 2; q++) {
                tile_nodes[2 * (tn_pos + q)] = (uint32_t)(c.node_base + P.tile_nodes[2 * q]);
                tile_nodes[2 * (tn_pos + q) + 1] = P.tile_nodes[2 * q + 1];
            }
            tn_pos += (int64_t)P.tile_nodes.size() / 2;
            std::memcpy(&lconn[4 * c.tet_base], P.lconn.data(), P.lconn.size());
            std::memcpy(&tile_inc[4 * c.tet_base], P.tile_inc.data(), P.tile_inc.size() * sizeof(uint16_t));
            for (int64_t t = 0; t < P.nslots; t++) {
                const float* o = &P.dmi[12 * t];
                const size_t q = (size_t)(c.tet_base + t);
                for (int e = 0; e < 4; e++) da[4 * q + e] = o[e];
                for (int e = 0; e < 4; e++) db[4 * q + e] = o[4 + e];
                dc[2 * q] = o[8];
                dc[2 * q + 1] = o[9];
            }
        }
        tile_tet_begin[nti] = (int)nt;
        tile_node_begin[nti] = (int)tn_pos;
        int* d_ttb; int* d_tnb; unsigned* d_tm; uint2* d_tn; uchar4* d_lc; ushort4* d_ti; float4 *d_da, *d_db;
        float2* d_dc; int* d_tc;
        float4 *d_pa = nullptr, *d_pb = nullptr; float2 *d_pc = nullptr, *d_fields = nullptr;
        if ((rc = balloc(A, &d_ttb, nti + 1)) || (rc = balloc(A, &d_tnb, nti + 1)) || (rc = balloc(A, &d_tm, nti)) ||
            (rc = balloc(A, &d_tn, ntn + ARRAY_PAD)) || (rc = balloc(A, &d_lc, ntp)) || (rc = balloc(A, &d_ti, ntp)) ||
            (rc = balloc(A, &d_da, ntp)) || (rc = balloc(A, &d_db, ntp)) || (rc = balloc(A, &d_dc, ntp)) ||
            (rc = balloc(A, &d_tc, nti)))
            return rc;
        if (b->model == MODEL_VP) {
            if ((rc = balloc(A, &d_pa, ntp)) || (rc = balloc(A, &d_pb, ntp)) || (rc = balloc(A, &d_pc, ntp)) ||
                (rc = balloc(A, &d_fields, ntp)))
                return rc;
        }
        BCUDA(cudaMemcpyAsync(d_ttb, tile_tet_begin.data(), tile_tet_begin.size() * sizeof(int), cudaMemcpyHostToDevice, st));
        BCUDA(cudaMemcpyAsync(d_tnb, tile_node_begin.data(), tile_node_begin.size() * sizeof(int), cudaMemcpyHostToDevice, st));
        BCUDA(cudaMemsetAsync(d_tn, 0, (ntn + ARRAY_PAD) * sizeof(uint2), st));
        if (nti > 0) {
            BCUDA(cudaMemcpyAsync(d_tm, tile_meta.data(), nti * sizeof(unsigned), cudaMemcpyHostToDevice, st));
            BCUDA(cudaMemcpyAsync(d_tc, tile_cell.data(), nti * sizeof(int), cudaMemcpyHostToDevice, st));
        }
        if (ntn > 0)
            BCUDA(cudaMemcpyAsync(d_tn, tile_nodes.data(), tile_nodes.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
        BCUDA(cudaMemcpyAsync(d_lc, lconn.data(), lconn.size(), cudaMemcpyHostToDevice, st));
        BCUDA(cudaMemcpyAsync(d_ti, tile_inc.data(), tile_inc.size() * sizeof(uint16_t), cudaMemcpyHostToDevice, st));
        BCUDA(cudaMemcpyAsync(d_da, da.data(), da.size() * sizeof(float), cudaMemcpyHostToDevice, st));
        BCUDA(cudaMemcpyAsync(d_db, db.data(), db.size() * sizeof(float), cudaMemcpyHostToDevice, st));
        BCUDA(cudaMemcpyAsync(d_dc, dc.data(), dc.size() * sizeof(float), cudaMemcpyHostToDevice, st));
        if (b->model == MODEL_VP) {
            BCUDA(cudaMemsetAsync(d_pa, 0, ntp * sizeof(float4), st));
            BCUDA(cudaMemsetAsync(d_pb, 0, ntp * sizeof(float4), st));
            BCUDA(cudaMemsetAsync(d_pc, 0, ntp * sizeof(float2), st));
            BCUDA(cudaMemsetAsync(d_fields, 0, ntp * sizeof(float2), st));
        }
        BCUDA(cudaStreamSynchronize(st));
        MeshDev& KM = K.mesh;
        KM = M;
        KM.nt = (int)nt;
        KM.ntiles = (int)nti;
        KM.tile_tets = tiles[g];
        KM.tile_base = (int)bk_tile_base[g];
        KM.tile_tet_begin = d_ttb;
        KM.tile_node_begin = d_tnb;
        KM.tile_nodes = d_tn;
        KM.tile_meta = d_tm;
        KM.lconn = d_lc;
        KM.tile_inc = d_ti;
        KM.dmi_a = d_da;
        KM.dmi_b = d_db;
        KM.dmi_c = d_dc;
        K.st = S;
        K.st.vp_a = d_pa;
        K.st.vp_b = d_pb;
        K.st.vp_c = d_pc;
        K.st.fields = d_fields;
        K.bd = B;
        K.bd.tile_cell = d_tc;
    }
    BCUDA(launch_advance_time(S, 0, B.fields_every, B.record_every, st));
    BCUDA(cudaStreamSynchronize(st));
    return NFX_OK;
}

int enqueue_batch_steps(nfx_batch* b, BatchDevice& D, int n) {
    for (int k = 0; k < n; k++) {
        for (BucketDev& K : D.buckets) {
            if (K.mesh.ntiles <= 0) continue;
            BCUDA(launch_tet_pass(K.mesh, K.st, K.bd, b->model, k, b->stream, true));
            if (b->has_si) BCUDA(launch_si_pass(K.mesh, K.st, K.bd, k, false, -1, b->stream));
        }
        BCUDA(launch_node_pass(D.mesh, D.st, D.bd, D.nblocks, k, NODE_UPDATE, -1, b->stream, true));
    }
    BCUDA(launch_advance_time(D.st, n, D.bd.fields_every, D.bd.record_every, b->stream));
    return NFX_OK;
}

int batch_step(nfx_batch* b, BatchDevice& D, int64_t nsteps) {
    int64_t left = nsteps;
    while (left >= BATCH_GRAPH_STEPS) {
        if (!D.graph) {
            cudaGraph_t g = nullptr;
            BCUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
            int rc = enqueue_batch_steps(b, D, BATCH_GRAPH_STEPS);
            cudaError_t e = cudaStreamEndCapture(b->stream, &g);
            if (rc != NFX_OK) {
                if (g) cudaGraphDestroy(g);
                return rc;
            }
            if (e != cudaSuccess) return bfail(NFX_ERR_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e));
            e = cudaGraphInstantiate(&D.graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return bfail(NFX_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
        }
        BCUDA(cudaGraphLaunch(D.graph, b->stream));
        left -= BATCH_GRAPH_STEPS;
    }
    if (left > 0) return enqueue_batch_steps(b, D, (int)left);
    return NFX_OK;
}

// Autotuner of one bucket: time a few steps of a representative sub-batch of the bucket's cells
// (cells at the size quantiles) for each candidate tile size and keep the fastest.
int autotune_bucket(nfx_batch* b, int g, const std::vector<int>& members, int& best) {
    std::vector<int> order(members);
    std::sort(order.begin(), order.end(), [&](int x, int y) { return b->cells[x].nt < b->cells[y].nt; });
    std::vector<int> sample;
    const int want = std::min<int>(8, (int)order.size());
    for (int q = 0; q < want; q++) {
        const int idx = (int)((q + 0.5) * order.size() / want);
        sample.push_back(order[std::min<int>(idx, (int)order.size() - 1)]);
    }
    std::sort(sample.begin(), sample.end());
    sample.erase(std::unique(sample.begin(), sample.end()), sample.end());
    const int candidates[3] = {64, 128, 256};
    float best_ms = 1e30f;
    best = DEFAULT_TILE_TETS;
    for (int tile : candidates) {
        int rc = build_plans(b, sample, tile);
        if (rc != NFX_OK) return rc;
        BatchDevice D;
        rc = build_device(b, sample, std::vector<int>(sample.size(), 0), {tile}, D);
        if (rc != NFX_OK) {
            D.release();
            return rc;
        }
        rc = enqueue_batch_steps(b, D, 3);  // warm-up
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0, b->stream);
        if (rc == NFX_OK) rc = enqueue_batch_steps(b, D, 10);
        cudaEventRecord(e1, b->stream);
        cudaError_t e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        D.release();
        if (rc != NFX_OK) return rc;
        if (e != cudaSuccess) return bfail(NFX_ERR_CUDA, std::string("autotune: ") + cudaGetErrorString(e));
        b->tuned.push_back(tile);
        b->tuned_ms.push_back(ms);
        b->tuned_bucket.push_back(g);
        if (ms < best_ms) {
            best_ms = ms;
            best = tile;
        }
    }
    return NFX_OK;
}

// rows produced by node passes at times in [t_begin, t_end] (row r is time r*every)
void note_batch_rows(nfx_batch* b, long long t_begin, long long t_end) {
    if (b->record_contact < 0 || b->record_every <= 0 || t_end < t_begin) return;
    const long long last = t_end / b->record_every;
    if (last * b->record_every >= t_begin) b->rows_written = std::max(b->rows_written, std::min(last + 1, b->max_rows));
}

int check_cell(nfx_batch* b, int cell) {
    if (!b) return bfail(NFX_ERR_ARG, "null batch");
    if (cell < 0 || cell >= (int)b->cells.size()) return bfail(NFX_ERR_ARG, "cell index out of range");
    return NFX_OK;
}

}  // namespace

extern "C" {

int nfx_batch_create(int device, int tile_tets, nfx_batch** out) {
    BARG(out, "out is null");
    *out = nullptr;
    BARG(tile_tets == 0 || tile_tets == 64 || tile_tets == 128 || tile_tets == 256 || tile_tets == 512,
         "tile size must be 0 (autotune), 64, 128, 256 or 512");
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) return bfail(NFX_ERR_NODEVICE, std::string("no CUDA device: ") + cudaGetErrorString(e));
    if (device < 0 || device >= count) return bfail(NFX_ERR_NODEVICE, "device id out of range");
    BCUDA(cudaSetDevice(device));
    nfx_batch* b = new nfx_batch();
    b->device = device;
    b->tile_tets = tile_tets;
    e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete b;
        return bfail(NFX_ERR_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
    }
    void* z = nullptr;
    e = cudaMalloc(&z, 2 * sizeof(long long));
    if (e != cudaSuccess) {
        cudaStreamDestroy(b->stream);
        delete b;
        return bfail(NFX_ERR_NOMEM, "cudaMalloc");
    }
    cudaMemset(z, 0, 2 * sizeof(long long));
    b->d_zero_meta = (long long*)z;
    *out = b;
    return NFX_OK;
}

int nfx_batch_destroy(nfx_batch* b) {
    if (!b) return NFX_OK;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    b->dev.release();
    if (b->d_zero_meta) cudaFree(b->d_zero_meta);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return NFX_OK;
}

int nfx_batch_add_cell(nfx_batch* b, int64_t np, int64_t nt, const double* points, const uint32_t* tets, int* cell) {
    BARG(b && points && tets, "null argument");
    if (b->finalized) return bfail(NFX_ERR_STATE, "batch already finalized");
    BARG(np > 0 && nt > 0, "empty mesh");
    CellHost c;
    c.np = np;
    c.nt = nt;
    c.points.assign(points, points + 3 * np);
    c.tets.assign(tets, tets + 4 * nt);
    b->cells.push_back(std::move(c));
    if (cell) *cell = (int)b->cells.size() - 1;
    return NFX_OK;
}

int nfx_batch_add_cell_like(nfx_batch* b, int src, int* cell) {
    int rc;
    if ((rc = check_cell(b, src)) != NFX_OK) return rc;
    if (b->finalized) return bfail(NFX_ERR_STATE, "batch already finalized");
    CellHost c;
    c.np = b->cells[src].np;
    c.nt = b->cells[src].nt;
    c.mesh_src = mesh_owner(b, src);
    b->cells.push_back(std::move(c));
    if (cell) *cell = (int)b->cells.size() - 1;
    return NFX_OK;
}

int nfx_batch_set_tetra(nfx_batch* b, int cell, int model, double E, double nu, double mr) {
    int rc;
    if ((rc = check_cell(b, cell)) != NFX_OK) return rc;
    if (b->finalized) return bfail(NFX_ERR_STATE, "batch already finalized");
    BARG(model == NFX_MODEL_MR || model == NFX_MODEL_SVK || model == NFX_MODEL_SVKK, "unknown elastic model");
    BARG(b->model < 0 || b->model == model, "all cells of a batch use one material model");
    BARG(std::isfinite(E) && std::isfinite(nu) && std::isfinite(mr) && nu != 0.5, "bad material parameter");
    const double mu = E / (2 * (1 + nu));
    MaterialDev& m = b->cells[cell].mat;
    m = MaterialDev{};
    m.model = model;
    m.mu1 = (float)(mr * mu);
    m.mu2 = (float)((1 - mr) * mu);
    m.kappa = (float)(E / (3 * (1 - 2 * nu)));
    m.mu = (float)mu;
    m.kp = (float)(nu / (1 - 2 * nu));
    b->cells[cell].has_mat = true;
    b->model = model;
    return NFX_OK;
}

int nfx_batch_set_viscoplastic(nfx_batch* b, int cell, const double* par) {
    int rc;
    if ((rc = check_cell(b, cell)) != NFX_OK) return rc;
    if (b->finalized) return bfail(NFX_ERR_STATE, "batch already finalized");
    BARG(par, "null parameters");
    BARG(b->model < 0 || b->model == MODEL_VP, "all cells of a batch use one material model");
    for (int k = 0; k < 8; k++) BARG(std::isfinite(par[k]), "non-finite viscoplastic parameter");
    BARG(par[4] > 0 && par[6] != 0, "yield stress must be positive and the hardening threshold non-zero");
    MaterialDev& m = b->cells[cell].mat;
    m = MaterialDev{};
    m.model = MODEL_VP;
    m.mu1 = (float)par[0];
    m.mu2 = (float)par[1];
    m.kappa = (float)par[2];
    m.flow_exp = (float)par[3];
    m.yield = (float)par[4];
    m.flow_rate = (float)par[5];
    m.hard_thr = (float)par[6];
    m.hard_exp = (float)par[7];
    b->cells[cell].has_mat = true;
    b->model = MODEL_VP;
    return NFX_OK;
}

int nfx_batch_add_contact(nfx_batch* b, int cell, int kind, double k, double radius, double p0, double v, double tmove,
                          int* id) {
    int rc;
    if ((rc = check_cell(b, cell)) != NFX_OK) return rc;
    if (b->finalized) return bfail(NFX_ERR_STATE, "batch already finalized");
    CellHost& c = b->cells[cell];
    BARG(c.n_contacts < MAX_CONTACTS, "at most 4 contacts per cell");
    BARG(kind == NFX_CONTACT_SUBSTRATE || kind == NFX_CONTACT_PLANE || kind == NFX_CONTACT_SPHERE ||
             kind == NFX_CONTACT_SPHERE_INTEGRAL,
         "unknown contact kind");
    BARG(std::isfinite(k) && std::isfinite(p0) && std::isfinite(v) && !std::isnan(tmove), "non-finite contact parameter");
    BARG((kind != NFX_CONTACT_SPHERE && kind != NFX_CONTACT_SPHERE_INTEGRAL) || radius > 0,
         "sphere radius must be positive");
    BARG(kind != NFX_CONTACT_SPHERE_INTEGRAL || c.si_contact < 0, "at most one integrated sphere contact per cell");
    ContactDev& C = c.c[c.n_contacts];
    C = ContactDev{};
    C.kind = kind;
    C.k = k;
    C.radius = radius;
    C.p0 = p0;
    C.v = v;
    C.tmove = tmove;
    if (id) *id = c.n_contacts;
    if (kind == NFX_CONTACT_SPHERE_INTEGRAL) {
        c.si_contact = c.n_contacts;
        b->has_si = true;
    }
    c.n_contacts++;
    return NFX_OK;
}

int nfx_batch_set_integrator(nfx_batch* b, int cell, double xi, int fix_top_bottom) {
    int rc;
    if ((rc = check_cell(b, cell)) != NFX_OK) return rc;
    if (b->finalized) return bfail(NFX_ERR_STATE, "batch already finalized");
    BARG(std::isfinite(xi) && xi > -2.0, "bad damping");
    b->cells[cell].xi = xi;
    b->cells[cell].fix_top_bottom = fix_top_bottom != 0;
    b->cells[cell].integrator = INTEGRATOR_VV;
    return NFX_OK;
}

int nfx_batch_set_integrator_lumped(nfx_batch* b, int cell, double xi, double density) {
    int rc;
    if ((rc = check_cell(b, cell)) != NFX_OK) return rc;
    if (b->finalized) return bfail(NFX_ERR_STATE, "batch already finalized");
    BARG(std::isfinite(xi) && xi > -2.0, "bad damping");
    BARG(std::isfinite(density) && density > 0, "density must be positive");
    CellHost& c = b->cells[cell];
    c.xi = xi;
    c.fix_top_bottom = false;
    c.integrator = INTEGRATOR_VV2;
    c.density = density;
    return NFX_OK;
}

int nfx_batch_set_record(nfx_batch* b, int contact, int64_t every, int64_t max_rows) {
    BARG(b, "null batch");
    if (b->finalized) return bfail(NFX_ERR_STATE, "batch already finalized");
    BARG(contact >= -1 && contact < MAX_CONTACTS, "contact index out of range");
    BARG(contact < 0 || (every > 0 && max_rows > 0), "every and max_rows must be positive");
    b->record_contact = contact;
    b->record_every = every;
    b->max_rows = max_rows;
    return NFX_OK;
}

int nfx_batch_finalize(nfx_batch* b) {
    const NvtxRange range("nfx_batch_finalize");
    BARG(b, "null batch");
    if (b->finalized) return bfail(NFX_ERR_STATE, "batch already finalized");
    BARG(!b->cells.empty(), "batch has no cells");
    for (size_t i = 0; i < b->cells.size(); i++)
        if (!b->cells[i].has_mat) return bfail(NFX_ERR_STATE, "cell " + std::to_string(i) + " has no material");
    BCUDA(cudaSetDevice(b->device));
    int rc;
    std::vector<int> all(b->cells.size());
    for (size_t i = 0; i < all.size(); i++) all[i] = (int)i;
    // buckets: one for every cell at a fixed tile size; by size class under the autotuner
    std::vector<int> bucket(all.size(), 0), tiles;
    if (b->tile_tets != 0) {
        tiles.push_back(b->tile_tets);
    } else {
        int present[MAX_BUCKETS] = {-1, -1, -1};
        for (size_t i = 0; i < all.size(); i++) present[size_class(b->cells[i].nt)] = 0;
        int ng = 0;
        for (int q = 0; q < MAX_BUCKETS; q++)
            if (present[q] == 0) present[q] = ng++;
        for (size_t i = 0; i < all.size(); i++) bucket[i] = present[size_class(b->cells[i].nt)];
        tiles.assign(ng, DEFAULT_TILE_TETS);
        b->tuned.clear();
        b->tuned_ms.clear();
        b->tuned_bucket.clear();
        for (int g = 0; g < ng; g++) {
            std::vector<int> members;
            for (size_t i = 0; i < all.size(); i++)
                if (bucket[i] == g) members.push_back((int)i);
            if ((rc = autotune_bucket(b, g, members, tiles[g])) != NFX_OK) return rc;
        }
    }
    for (int g = 0; g < (int)tiles.size(); g++) {
        std::vector<int> members;
        for (size_t i = 0; i < all.size(); i++)
            if (bucket[i] == g) members.push_back((int)i);
        if ((rc = build_plans(b, members, tiles[g])) != NFX_OK) return rc;
    }
    if ((rc = build_device(b, all, bucket, tiles, b->dev)) != NFX_OK) return rc;
    // the tile size reported for the batch: that of the bucket holding the most tetrahedra
    int64_t most = -1;
    for (const BucketDev& K : b->dev.buckets)
        if (K.tets > most) {
            most = K.tets;
            b->tile_tets = K.tile_tets;
        }
    // only the maps for readback are kept on the host
    for (auto& c : b->cells) {
        MeshPlan& P = *c.plan;
        P.lconn = {};
        P.tile_inc = {};
        P.dmi = {};
        P.tile_nodes = {};
        P.Xh = {};
        P.Xl = {};
        c.points = {};
        c.tets = {};
    }
    b->finalized = true;
    b->time = 0;
    return NFX_OK;
}

int nfx_batch_step(nfx_batch* b, int64_t nsteps) {
    const NvtxRange range("nfx_batch_step");
    BARG(b, "null batch");
    if (!b->finalized) return bfail(NFX_ERR_STATE, "call nfx_batch_finalize first");
    BARG(nsteps >= 0, "negative step count");
    BCUDA(cudaSetDevice(b->device));
    const long long t0 = b->time;
    int rc = batch_step(b, b->dev, nsteps);
    if (rc == NFX_OK) {
        b->time += nsteps;
        if (nsteps > 0) note_batch_rows(b, t0, b->time - 1);
    }
    return rc;
}

int nfx_batch_time_steps(nfx_batch* b, int64_t nsteps, float* ms) {
    BARG(b && ms, "null argument");
    if (!b->finalized) return bfail(NFX_ERR_STATE, "call nfx_batch_finalize first");
    BCUDA(cudaSetDevice(b->device));
    cudaEvent_t e0, e1;
    BCUDA(cudaEventCreate(&e0));
    BCUDA(cudaEventCreate(&e1));
    cudaEventRecord(e0, b->stream);
    int rc = batch_step(b, b->dev, nsteps);
    cudaEventRecord(e1, b->stream);
    cudaError_t e = cudaEventSynchronize(e1);
    float t = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != NFX_OK) return rc;
    if (e != cudaSuccess) return bfail(NFX_ERR_CUDA, std::string("event timing: ") + cudaGetErrorString(e));
    const long long t0 = b->time;
    b->time += nsteps;
    if (nsteps > 0) note_batch_rows(b, t0, b->time - 1);
    *ms = t;
    return NFX_OK;
}

int nfx_batch_record_now(nfx_batch* b) {
    BARG(b, "null batch");
    if (!b->finalized) return bfail(NFX_ERR_STATE, "call nfx_batch_finalize first");
    BCUDA(cudaSetDevice(b->device));
    if (b->has_si && b->record_contact >= 0)
        for (BucketDev& K : b->dev.buckets)
            if (K.mesh.ntiles > 0) BCUDA(launch_si_pass(K.mesh, K.st, K.bd, 0, true, b->record_contact, b->stream));
    BCUDA(launch_node_pass(b->dev.mesh, b->dev.st, b->dev.bd, b->dev.nblocks, 0, NODE_READOUT_ROW, -1, b->stream));
    note_batch_rows(b, b->time, b->time);
    return NFX_OK;
}

int nfx_batch_indenter_force(nfx_batch* b, int contact, double* out) {
    BARG(b && out, "null argument");
    BARG(contact >= 0 && contact < MAX_CONTACTS, "contact id out of range");
    if (!b->finalized) return bfail(NFX_ERR_STATE, "call nfx_batch_finalize first");
    BCUDA(cudaSetDevice(b->device));
    if (b->has_si)
        for (BucketDev& K : b->dev.buckets)
            if (K.mesh.ntiles > 0) BCUDA(launch_si_pass(K.mesh, K.st, K.bd, 0, true, contact, b->stream));
    BCUDA(launch_node_pass(b->dev.mesh, b->dev.st, b->dev.bd, b->dev.nblocks, 0, NODE_READOUT_VALUE, contact, b->stream));
    BCUDA(cudaMemcpyAsync(out, b->dev.st.force_out, b->cells.size() * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    BCUDA(cudaStreamSynchronize(b->stream));
    return NFX_OK;
}

int nfx_batch_get_curve(nfx_batch* b, int cell, double* rows, int64_t max_rows, int64_t* n_rows) {
    int rc;
    if ((rc = check_cell(b, cell)) != NFX_OK) return rc;
    BARG(n_rows && (max_rows == 0 || rows), "bad row buffer");
    if (!b->finalized) return bfail(NFX_ERR_STATE, "call nfx_batch_finalize first");
    BCUDA(cudaSetDevice(b->device));
    const long long avail = b->rows_written;
    const long long n = std::min<long long>(avail, max_rows);
    if (n > 0)
        BCUDA(cudaMemcpyAsync(rows, b->dev.bd.curves + 3 * (size_t)cell * b->max_rows, 3 * (size_t)n * sizeof(double),
                              cudaMemcpyDeviceToHost, b->stream));
    BCUDA(cudaStreamSynchronize(b->stream));
    *n_rows = avail;
    return NFX_OK;
}

int nfx_batch_get_points(nfx_batch* b, int cell, double* out) {
    int rc;
    if ((rc = check_cell(b, cell)) != NFX_OK) return rc;
    BARG(out, "null out");
    if (!b->finalized) return bfail(NFX_ERR_STATE, "call nfx_batch_finalize first");
    BCUDA(cudaSetDevice(b->device));
    const CellHost& c = b->cells[cell];
    const size_t np = (size_t)c.np;
    std::vector<float> xh(4 * np), xl(4 * np), ua(4 * np), ub(2 * np);
    const size_t off = (size_t)c.node_base;
    const MeshDev& M = b->dev.mesh;
    BCUDA(cudaMemcpyAsync(xh.data(), M.Xh + off, np * sizeof(float4), cudaMemcpyDeviceToHost, b->stream));
    BCUDA(cudaMemcpyAsync(xl.data(), M.Xl + off, np * sizeof(float4), cudaMemcpyDeviceToHost, b->stream));
    BCUDA(cudaMemcpyAsync(ua.data(), b->dev.st.ua + off, np * sizeof(float4), cudaMemcpyDeviceToHost, b->stream));
    BCUDA(cudaMemcpyAsync(ub.data(), b->dev.st.ub + off, np * sizeof(float2), cudaMemcpyDeviceToHost, b->stream));
    BCUDA(cudaStreamSynchronize(b->stream));
    for (size_t i = 0; i < np; i++) {
        const int64_t u = c.plan->node_user[i];
        const float lo[3] = {ua[4 * i + 3], ub[2 * i], ub[2 * i + 1]};
        for (int d = 0; d < 3; d++)
            out[d * np + u] = ((double)xh[4 * i + d] + (double)xl[4 * i + d]) + ((double)ua[4 * i + d] + (double)lo[d]);
    }
    return NFX_OK;
}

int nfx_batch_set_points(nfx_batch* b, int cell, const double* in) {
    int rc;
    if ((rc = check_cell(b, cell)) != NFX_OK) return rc;
    BARG(in, "null input");
    if (!b->finalized) return bfail(NFX_ERR_STATE, "call nfx_batch_finalize first");
    const CellHost& c = b->cells[cell];
    const size_t np = (size_t)c.np;
    for (size_t i = 0; i < 3 * np; i++) BARG(std::isfinite(in[i]), "non-finite position");
    BCUDA(cudaSetDevice(b->device));
    std::vector<float> xh(4 * np), xl(4 * np), ua(4 * np, 0.f), ub(2 * np, 0.f);
    const size_t off = (size_t)c.node_base;
    const MeshDev& M = b->dev.mesh;
    BCUDA(cudaMemcpyAsync(xh.data(), M.Xh + off, np * sizeof(float4), cudaMemcpyDeviceToHost, b->stream));
    BCUDA(cudaMemcpyAsync(xl.data(), M.Xl + off, np * sizeof(float4), cudaMemcpyDeviceToHost, b->stream));
    BCUDA(cudaStreamSynchronize(b->stream));
    // the displacement x - X as float hi + lo, as the single-cell setter forms it on the device
    for (size_t i = 0; i < np; i++) {
        const int64_t u = c.plan->node_user[i];
        float lo[3];
        for (int d = 0; d < 3; d++) {
            const double dx = (in[d * np + u] - (double)xh[4 * i + d]) - (double)xl[4 * i + d];
            const float h = (float)dx;
            ua[4 * i + d] = h;
            lo[d] = (float)(dx - (double)h);
        }
        ua[4 * i + 3] = lo[0];
        ub[2 * i] = lo[1];
        ub[2 * i + 1] = lo[2];
    }
    BCUDA(cudaMemcpyAsync(b->dev.st.ua + off, ua.data(), np * sizeof(float4), cudaMemcpyHostToDevice, b->stream));
    BCUDA(cudaMemcpyAsync(b->dev.st.ub + off, ub.data(), np * sizeof(float2), cudaMemcpyHostToDevice, b->stream));
    BCUDA(cudaStreamSynchronize(b->stream));
    return NFX_OK;
}

int nfx_batch_status(nfx_batch* b, uint32_t* flags, int clear) {
    BARG(b && flags, "null argument");
    if (!b->finalized) return bfail(NFX_ERR_STATE, "call nfx_batch_finalize first");
    BCUDA(cudaSetDevice(b->device));
    unsigned h = 0;
    BCUDA(cudaMemcpyAsync(&h, b->dev.d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, b->stream));
    if (clear) BCUDA(cudaMemsetAsync(b->dev.d_status, 0, sizeof(unsigned), b->stream));
    BCUDA(cudaStreamSynchronize(b->stream));
    *flags = h;
    return NFX_OK;
}

int nfx_batch_cell_status(nfx_batch* b, uint32_t* flags, int clear) {
    BARG(b && flags, "null argument");
    if (!b->finalized) return bfail(NFX_ERR_STATE, "call nfx_batch_finalize first");
    BCUDA(cudaSetDevice(b->device));
    const size_t n = b->cells.size();
    BCUDA(cudaMemcpyAsync(flags, b->dev.bd.cell_status, n * sizeof(unsigned), cudaMemcpyDeviceToHost, b->stream));
    if (clear) BCUDA(cudaMemsetAsync(b->dev.bd.cell_status, 0, n * sizeof(unsigned), b->stream));
    BCUDA(cudaStreamSynchronize(b->stream));
    return NFX_OK;
}

int nfx_batch_info(nfx_batch* b, int64_t* cells, int64_t* tets, int64_t* nodes, int* tile_tets) {
    BARG(b && cells && tets && nodes && tile_tets, "null argument");
    int64_t nt = 0, np = 0;
    for (auto& c : b->cells) {
        nt += c.nt;
        np += c.np;
    }
    *cells = (int64_t)b->cells.size();
    *tets = nt;
    *nodes = np;
    *tile_tets = b->tile_tets;
    return NFX_OK;
}

int nfx_batch_tuning(nfx_batch* b, int* tiles, float* ms, int max_n, int* n) {
    BARG(b && n, "null argument");
    const int k = (int)b->tuned.size();
    for (int i = 0; i < std::min(k, max_n); i++) {
        if (tiles) tiles[i] = b->tuned[i];
        if (ms) ms[i] = b->tuned_ms[i];
    }
    *n = k;
    return NFX_OK;
}

int nfx_batch_buckets(nfx_batch* b, int max_n, int* n, int* tile_tets, int64_t* cells, int64_t* tets) {
    BARG(b && n, "null argument");
    if (!b->finalized) return bfail(NFX_ERR_STATE, "call nfx_batch_finalize first");
    const int k = (int)b->dev.buckets.size();
    for (int i = 0; i < std::min(k, max_n); i++) {
        const BucketDev& K = b->dev.buckets[i];
        if (tile_tets) tile_tets[i] = K.tile_tets;
        if (cells) cells[i] = K.cells;
        if (tets) tets[i] = K.tets;
    }
    *n = k;
    return NFX_OK;
}

}  // extern "C"
