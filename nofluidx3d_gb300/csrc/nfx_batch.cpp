// Batched cells (C ABI nfx_batch_*): many independent cells of uneven size and material advance
// together. Each cell's mesh gets its own plan (reordering, tiles, Dm^-1), built on host threads;
// the plans are concatenated into one set of device arrays. Every cell's nodes occupy whole node
// blocks, so the node pass maps a block to one cell; every tile belongs to one cell, so the
// element pass maps a tile to one cell. One element-pass launch and one node-pass launch advance
// all cells per step, and chunks of steps are captured as a CUDA graph. The reference has no
// batched mode: its equivalent is one Simulation per cell (nofluidx3d/Simulation.py:35).
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

// Device arrays of one built batch (a full batch, or a sub-batch the autotuner times).
struct BatchDevice {
    std::vector<void*> allocs;
    MeshDev mesh{};
    StateDev st{};
    BatchDev bd{};
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
    std::vector<int> tuned;    // tile sizes the autotuner tried
    std::vector<float> tuned_ms;
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

// Concatenate the plans of `which` into device arrays (zeroed state).
int build_device(nfx_batch* b, const std::vector<int>& which, int tile_tets, BatchDevice& D) {
    D.release();
    int64_t np = 0, nt = 0, ntiles = 0, nblocks = 0, ntn = 0;
    for (int ci : which) {
        CellHost& c = b->cells[ci];
        c.node_base = np;
        c.tet_base = nt;
        c.tile_base = ntiles;
        c.block_base = nblocks;
        c.nblocks = (c.np + NODE_BLOCK - 1) / NODE_BLOCK;
        np += c.nblocks * NODE_BLOCK;  // whole blocks per cell
        nt += c.plan->nslots;  // tetra slots (whole tiles)
        ntiles += c.plan->ntiles;
        nblocks += c.nblocks;
        ntn += (int64_t)c.plan->tile_nodes.size() / 2;
    }
    if (np > 0x7fffffff || nt > 0x7fffffff) return bfail(NFX_ERR_ARG, "batch too large");
    const size_t ntp = (size_t)nt + ARRAY_PAD;
    std::vector<int> tile_tet_begin(ntiles + 1), tile_node_begin(ntiles + 1), tile_cell(ntiles), block_cell(nblocks);
    std::vector<unsigned> tile_meta(ntiles);
    std::vector<uint32_t> tile_nodes(2 * (size_t)ntn);
    std::vector<uint8_t> lconn(4 * ntp, 0);
    std::vector<uint16_t> tile_inc(4 * ntp, 0);
    std::vector<float> da(4 * ntp, 0.f), db(4 * ntp, 0.f), dc(2 * ntp, 0.f);
    std::vector<float> Xh(4 * (size_t)np, 0.f), Xl(4 * (size_t)np, 0.f);
    std::vector<CellDev> cells(which.size());
    int64_t tn_pos = 0;
    for (size_t k = 0; k < which.size(); k++) {
        CellHost& c = b->cells[which[k]];
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
            const size_t g = (size_t)(c.tet_base + t);
            for (int q = 0; q < 4; q++) da[4 * g + q] = o[q];
            for (int q = 0; q < 4; q++) db[4 * g + q] = o[4 + q];
            dc[2 * g] = o[8];
            dc[2 * g + 1] = o[9];
        }
        std::memcpy(&Xh[4 * c.node_base], P.Xh.data(), P.Xh.size() * sizeof(float));
        std::memcpy(&Xl[4 * c.node_base], P.Xl.data(), P.Xl.size() * sizeof(float));
        for (int64_t q = 0; q < c.nblocks; q++) block_cell[c.block_base + q] = (int)k;
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
        C.tile_begin = (int)c.tile_base;
        C.tile_end = (int)(c.tile_base + P.ntiles);
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
    tile_tet_begin[ntiles] = (int)nt;
    tile_node_begin[ntiles] = (int)tn_pos;

    auto& A = D.allocs;
    int* d_ttb; int* d_tnb; unsigned* d_tm; uint2* d_tn; uchar4* d_lc; ushort4* d_ti; float4 *d_da, *d_db; float2* d_dc;
    float4 *d_xh, *d_xl, *d_uh, *d_ul, *d_v, *d_fo; unsigned long long* d_fa; double* d_part; double* d_fout;
    double* d_tpart;
    CellDev* d_cells; int *d_tc, *d_bc; unsigned* d_cc; unsigned* d_cst; double* d_curves = nullptr;
    float4 *d_pa = nullptr, *d_pb = nullptr; float2 *d_pc = nullptr, *d_fields = nullptr;
    int rc;
    const size_t rows = (size_t)std::max<long long>(b->max_rows, 1);
    if ((rc = balloc(A, &d_ttb, ntiles + 1)) || (rc = balloc(A, &d_tnb, ntiles + 1)) ||
        (rc = balloc(A, &d_tm, ntiles)) || (rc = balloc(A, &d_tn, ntn + ARRAY_PAD)) || (rc = balloc(A, &d_lc, ntp)) || (rc = balloc(A, &d_ti, ntp)) ||
        (rc = balloc(A, &d_da, ntp)) || (rc = balloc(A, &d_db, ntp)) || (rc = balloc(A, &d_dc, ntp)) ||
        (rc = balloc(A, &d_xh, np)) || (rc = balloc(A, &d_xl, np)) || (rc = balloc(A, &d_uh, np)) ||
        (rc = balloc(A, &d_ul, np)) || (rc = balloc(A, &d_v, np)) || (rc = balloc(A, &d_fo, np)) ||
        (rc = balloc(A, &d_fa, 3 * (size_t)np)) || (rc = balloc(A, &d_part, nblocks)) || (rc = balloc(A, &d_fout, cells.size())) ||
        (rc = balloc(A, &d_tpart, ntiles)) ||
        (rc = balloc(A, &d_cells, cells.size())) || (rc = balloc(A, &d_tc, ntiles)) || (rc = balloc(A, &d_bc, nblocks)) ||
        (rc = balloc(A, &d_cc, cells.size())) || (rc = balloc(A, &d_cst, cells.size())) ||
        (rc = balloc(A, &d_curves, 3 * rows * cells.size())) ||
        (rc = balloc(A, &D.d_clock, 1)) || (rc = balloc(A, &D.d_status, 1)))
        return rc;
    if (b->model == MODEL_VP) {
        if ((rc = balloc(A, &d_pa, ntp)) || (rc = balloc(A, &d_pb, ntp)) || (rc = balloc(A, &d_pc, ntp)) ||
            (rc = balloc(A, &d_fields, ntp)))
            return rc;
    }
    cudaStream_t st = b->stream;
    BCUDA(cudaMemcpyAsync(d_ttb, tile_tet_begin.data(), tile_tet_begin.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    BCUDA(cudaMemcpyAsync(d_tnb, tile_node_begin.data(), tile_node_begin.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    BCUDA(cudaMemsetAsync(d_tn, 0, (ntn + ARRAY_PAD) * sizeof(uint2), st));
    BCUDA(cudaMemcpyAsync(d_tm, tile_meta.data(), tile_meta.size() * sizeof(unsigned), cudaMemcpyHostToDevice, st));
    BCUDA(cudaMemcpyAsync(d_tn, tile_nodes.data(), tile_nodes.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    BCUDA(cudaMemcpyAsync(d_lc, lconn.data(), lconn.size(), cudaMemcpyHostToDevice, st));
    BCUDA(cudaMemcpyAsync(d_ti, tile_inc.data(), tile_inc.size() * sizeof(uint16_t), cudaMemcpyHostToDevice, st));
    BCUDA(cudaMemcpyAsync(d_da, da.data(), da.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    BCUDA(cudaMemcpyAsync(d_db, db.data(), db.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    BCUDA(cudaMemcpyAsync(d_dc, dc.data(), dc.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    BCUDA(cudaMemcpyAsync(d_xh, Xh.data(), Xh.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    BCUDA(cudaMemcpyAsync(d_xl, Xl.data(), Xl.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    for (float4* z : {d_uh, d_ul, d_v, d_fo}) BCUDA(cudaMemsetAsync(z, 0, (size_t)np * sizeof(float4), st));
    BCUDA(cudaMemsetAsync(d_fa, 0, 3 * (size_t)np * sizeof(unsigned long long), st));
    BCUDA(cudaMemcpyAsync(d_cells, cells.data(), cells.size() * sizeof(CellDev), cudaMemcpyHostToDevice, st));
    BCUDA(cudaMemcpyAsync(d_tc, tile_cell.data(), tile_cell.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    BCUDA(cudaMemcpyAsync(d_bc, block_cell.data(), block_cell.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    BCUDA(cudaMemsetAsync(d_cc, 0, cells.size() * sizeof(unsigned), st));
    BCUDA(cudaMemsetAsync(d_cst, 0, cells.size() * sizeof(unsigned), st));
    BCUDA(cudaMemsetAsync(d_curves, 0, 3 * rows * cells.size() * sizeof(double), st));
    BCUDA(cudaMemsetAsync(D.d_clock, 0, sizeof(StepClock), st));
    BCUDA(cudaMemsetAsync(D.d_status, 0, sizeof(unsigned), st));
    if (b->model == MODEL_VP) {
        BCUDA(cudaMemsetAsync(d_pa, 0, ntp * sizeof(float4), st));
        BCUDA(cudaMemsetAsync(d_pb, 0, ntp * sizeof(float4), st));
        BCUDA(cudaMemsetAsync(d_pc, 0, ntp * sizeof(float2), st));
        BCUDA(cudaMemsetAsync(d_fields, 0, ntp * sizeof(float2), st));
    }
    BCUDA(cudaStreamSynchronize(st));
    MeshDev& M = D.mesh;
    M.np = (int)np;
    M.nt = (int)nt;
    M.ntiles = (int)ntiles;
    M.tile_tets = tile_tets;
    M.tile_tet_begin = d_ttb;
    M.tile_node_begin = d_tnb;
    M.tile_nodes = d_tn;
    M.tile_meta = d_tm;
    M.lconn = d_lc;
    M.tile_inc = d_ti;
    M.dmi_a = d_da;
    M.dmi_b = d_db;
    M.dmi_c = d_dc;
    M.Xh = d_xh;
    M.Xl = d_xl;
    StateDev& S = D.st;
    S = StateDev{};
    S.uh = d_uh;
    S.ul = d_ul;
    S.v = d_v;
    S.fo = d_fo;
    S.facc = d_fa;
    S.vp_a = d_pa;
    S.vp_b = d_pb;
    S.vp_c = d_pc;
    S.fields = d_fields;
    S.status = D.d_status;
    S.clock = D.d_clock;
    S.partials = d_part;
    S.tile_partials = d_tpart;
    S.force_out = d_fout;
    BatchDev& B = D.bd;
    B.cells = d_cells;
    B.tile_cell = d_tc;
    B.block_cell = d_bc;
    B.cell_counter = d_cc;
    B.cell_status = d_cst;
    B.curves = d_curves;
    B.record_every = b->record_contact >= 0 ? b->record_every : 0;
    B.max_rows = b->max_rows;
    B.fields_every = b->record_every;
    D.nblocks = (int)nblocks;
    BCUDA(launch_advance_time(S, 0, B.fields_every, B.record_every, st));
    BCUDA(cudaStreamSynchronize(st));
    return NFX_OK;
}

int enqueue_batch_steps(nfx_batch* b, BatchDevice& D, int n) {
    for (int k = 0; k < n; k++) {
        BCUDA(launch_tet_pass(D.mesh, D.st, D.bd, b->model, k, b->stream));
        if (b->has_si) BCUDA(launch_si_pass(D.mesh, D.st, D.bd, k, false, -1, b->stream));
        BCUDA(launch_node_pass(D.mesh, D.st, D.bd, D.nblocks, k, NODE_UPDATE, -1, b->stream));
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

// Autotuner: time a few steps of a representative sub-batch (cells at the size quantiles) for
// each candidate tile size and keep the fastest per tetra.
int autotune(nfx_batch* b, int& best) {
    std::vector<int> order(b->cells.size());
    for (size_t i = 0; i < order.size(); i++) order[i] = (int)i;
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
    best = 128;
    b->tuned.clear();
    b->tuned_ms.clear();
    for (int tile : candidates) {
        int rc = build_plans(b, sample, tile);
        if (rc != NFX_OK) return rc;
        BatchDevice D;
        rc = build_device(b, sample, tile, D);
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
    BARG(b, "null batch");
    if (b->finalized) return bfail(NFX_ERR_STATE, "batch already finalized");
    BARG(!b->cells.empty(), "batch has no cells");
    for (size_t i = 0; i < b->cells.size(); i++)
        if (!b->cells[i].has_mat) return bfail(NFX_ERR_STATE, "cell " + std::to_string(i) + " has no material");
    BCUDA(cudaSetDevice(b->device));
    int tile = b->tile_tets;
    int rc;
    if (tile == 0 && (rc = autotune(b, tile)) != NFX_OK) return rc;
    b->tile_tets = tile;
    std::vector<int> all(b->cells.size());
    for (size_t i = 0; i < all.size(); i++) all[i] = (int)i;
    if ((rc = build_plans(b, all, tile)) != NFX_OK) return rc;
    if ((rc = build_device(b, all, tile, b->dev)) != NFX_OK) return rc;
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
        BCUDA(launch_si_pass(b->dev.mesh, b->dev.st, b->dev.bd, 0, true, b->record_contact, b->stream));
    BCUDA(launch_node_pass(b->dev.mesh, b->dev.st, b->dev.bd, b->dev.nblocks, 0, NODE_READOUT_ROW, -1, b->stream));
    note_batch_rows(b, b->time, b->time);
    return NFX_OK;
}

int nfx_batch_indenter_force(nfx_batch* b, int contact, double* out) {
    BARG(b && out, "null argument");
    BARG(contact >= 0 && contact < MAX_CONTACTS, "contact id out of range");
    if (!b->finalized) return bfail(NFX_ERR_STATE, "call nfx_batch_finalize first");
    BCUDA(cudaSetDevice(b->device));
    if (b->has_si) BCUDA(launch_si_pass(b->dev.mesh, b->dev.st, b->dev.bd, 0, true, contact, b->stream));
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
    std::vector<float> xh(4 * np), xl(4 * np), uh(4 * np), ul(4 * np);
    const size_t off = (size_t)c.node_base;
    const MeshDev& M = b->dev.mesh;
    BCUDA(cudaMemcpyAsync(xh.data(), M.Xh + off, np * sizeof(float4), cudaMemcpyDeviceToHost, b->stream));
    BCUDA(cudaMemcpyAsync(xl.data(), M.Xl + off, np * sizeof(float4), cudaMemcpyDeviceToHost, b->stream));
    BCUDA(cudaMemcpyAsync(uh.data(), b->dev.st.uh + off, np * sizeof(float4), cudaMemcpyDeviceToHost, b->stream));
    BCUDA(cudaMemcpyAsync(ul.data(), b->dev.st.ul + off, np * sizeof(float4), cudaMemcpyDeviceToHost, b->stream));
    BCUDA(cudaStreamSynchronize(b->stream));
    for (size_t i = 0; i < np; i++) {
        const int64_t u = c.plan->node_user[i];
        for (int d = 0; d < 3; d++)
            out[d * np + u] = ((double)xh[4 * i + d] + (double)xl[4 * i + d]) + ((double)uh[4 * i + d] + (double)ul[4 * i + d]);
    }
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

}  // extern "C"
