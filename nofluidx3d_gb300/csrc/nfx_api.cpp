// C ABI (include/nfx.h) of the GB300 tetra-mesh step: handle lifecycle, uploads, the step
// loop (CUDA-graph chunks) and conversions between the user's layout and the device state.
#include "../../include/nfx.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "nfx_internal.h"

using namespace nfx;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

#define CUDA_TRY(expr)                                                                              \
    do {                                                                                            \
        cudaError_t e_ = (expr);                                                                    \
        if (e_ != cudaSuccess) return fail(NFX_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define CHECK_ARG(cond, msg)                     \
    do {                                         \
        if (!(cond)) return fail(NFX_ERR_ARG, msg); \
    } while (0)

constexpr int GRAPH_STEPS = 100;  // steps per captured CUDA graph chunk

}  // namespace

void nfx::set_error(const std::string& msg) { g_err = msg; }

struct nfx_sim {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool have_mesh = false;
    bool have_material = false;
    MeshPlan plan;
    std::vector<void*> mesh_allocs;  // freed on re-mesh
    MeshDev mesh{};
    StateDev st{};
    // The simulation's parameters: a one-cell table the kernels read from device memory. The
    // host copy is uploaded in stream order before the next launch after any change.
    CellDev cell{};
    CellDev* d_cell = nullptr;
    bool cell_dirty = true;
    int nblocks = 0;                 // node blocks
    long long record_every = 0, max_rows = 0, fields_every = 0;
    long long* d_node_user = nullptr;
    double* d_stage = nullptr;
    // Per-step position tables of the contacts, two buffers per contact: a new table goes into
    // the buffer the enqueued steps do not read, and the cell table is repointed in stream order.
    // ev_table[c][k] marks the end of the work that may read buffer k (recorded when the cell
    // table moves away from it); a buffer is rewritten only after its event, so refilling a table
    // never drains the step stream.
    double* d_tables[MAX_CONTACTS][2] = {};
    long long* d_meta[MAX_CONTACTS][2] = {};
    long long table_cap[MAX_CONTACTS][2] = {};
    int table_cur[MAX_CONTACTS] = {0, 0, 0, 0};
    cudaEvent_t ev_table[MAX_CONTACTS][2] = {};
    bool ev_table_set[MAX_CONTACTS][2] = {};
    // fixed-size control block
    unsigned* d_status = nullptr;
    StepClock* d_clock = nullptr;
    unsigned* d_counter = nullptr;
    double* d_force_out = nullptr;
    double* d_curve = nullptr;
    long long curve_rows = 0;
    long long rows_written = 0;  // rows recorded so far (row r is time r*every)
    long long time = 0;          // host mirror of the device time
    cudaGraphExec_t graph = nullptr;
    bool graph_valid = false;
    int tile_tets = DEFAULT_TILE_TETS;     // tetrahedra per tile (64, 128, 256 or 512)
    // asynchronous output snapshots (nfx_snapshot): positions staged on the step stream, copied
    // to the host on a second stream while later steps run
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_snap = nullptr, ev_copy = nullptr;
    double* d_snap = nullptr;  // 3 * np doubles, allocated with the first snapshot of a mesh
    bool snap_pending = false;
};

namespace {

int set_device(nfx_sim* s) {
    CUDA_TRY(cudaSetDevice(s->device));
    return NFX_OK;
}

template <class T>
int dalloc(nfx_sim* /*s*/, T** p, size_t count, std::vector<void*>* owner) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
    if (e != cudaSuccess) return fail(NFX_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    *p = (T*)q;
    if (owner) owner->push_back(q);
    return NFX_OK;
}

// Waits for the copies of the last snapshot (before its staging or the curve buffer is freed or
// reset).
void snapshot_drain(nfx_sim* s) {
    if (s->snap_pending) {
        cudaEventSynchronize(s->ev_copy);
        s->snap_pending = false;
    }
}

void free_mesh(nfx_sim* s) {
    snapshot_drain(s);
    if (s->d_snap) cudaFree(s->d_snap);
    s->d_snap = nullptr;
    for (void* p : s->mesh_allocs) cudaFree(p);
    s->mesh_allocs.clear();
    s->mesh = MeshDev{};
    StateDev keep = s->st;
    s->st = StateDev{};
    s->st.status = keep.status;
    s->st.clock = keep.clock;
    s->st.force_out = keep.force_out;
    s->d_node_user = nullptr;
    s->d_stage = nullptr;
    s->have_mesh = false;
}

// Kernel view of the one-cell table (no tile or block maps: everything is cell 0).
BatchDev table_view(const nfx_sim* s) {
    BatchDev b{};
    b.cells = s->d_cell;
    b.cell_counter = s->d_counter;
    b.curves = s->d_curve;
    b.record_every = s->record_every;
    b.max_rows = s->max_rows;
    b.fields_every = s->fields_every;
    return b;
}

void invalidate_graph(nfx_sim* s) {
    if (s->graph) cudaGraphExecDestroy(s->graph);
    s->graph = nullptr;
    s->graph_valid = false;
}

int require_ready(nfx_sim* s) {
    if (!s) return fail(NFX_ERR_ARG, "null handle");
    if (!s->have_mesh) return fail(NFX_ERR_STATE, "no mesh: call nfx_set_mesh first");
    if (!s->have_material) return fail(NFX_ERR_STATE, "no material: call nfx_set_tetra or nfx_set_viscoplastic first");
    return NFX_OK;
}

// Upload the parameter table if it changed (stream-ordered: launches already enqueued read the
// old values, later ones the new). Pageable source: the copy has taken the bytes on return.
int upload_cell(nfx_sim* s) {
    if (!s->cell_dirty) return NFX_OK;
    CUDA_TRY(cudaMemcpyAsync(s->d_cell, &s->cell, sizeof(CellDev), cudaMemcpyHostToDevice, s->stream));
    s->cell_dirty = false;
    return NFX_OK;
}

// Element pass launch: one CTA per tile (pdl: as a dependent launch, inside a run of steps).
cudaError_t launch_elem(nfx_sim* s, int k, bool pdl = false) {
    return launch_tet_pass(s->mesh, s->st, table_view(s), s->cell.mat.model, k, s->stream, pdl);
}

cudaError_t launch_nodes(nfx_sim* s, int k, int mode, int readout_contact, bool pdl = false) {
    return launch_node_pass(s->mesh, s->st, table_view(s), s->nblocks, k, mode, readout_contact, s->stream, pdl);
}

// The integrated sphere contact's own tile pass, when the cell has one.
cudaError_t launch_si(nfx_sim* s, int k) {
    if (s->cell.si_contact < 0) return cudaSuccess;
    return launch_si_pass(s->mesh, s->st, table_view(s), k, false, -1, s->stream);
}

// Before a readout of contact `contact` between steps: the integrated sphere's tile partials.
cudaError_t prepare_readout(nfx_sim* s, int contact) {
    if (contact < 0 || contact != s->cell.si_contact) return cudaSuccess;
    return launch_si_pass(s->mesh, s->st, table_view(s), 0, true, contact, s->stream);
}

int enqueue_steps(nfx_sim* s, int n) {
    for (int k = 0; k < n; k++) {
        CUDA_TRY(launch_elem(s, k, true));                    // programmatic dependent launches
        CUDA_TRY(launch_si(s, k));
        CUDA_TRY(launch_nodes(s, k, NODE_UPDATE, -1, true));
    }
    CUDA_TRY(launch_advance_time(s->st, n, s->fields_every, s->record_every, s->stream));
    return NFX_OK;
}

int build_graph(nfx_sim* s) {
    invalidate_graph(s);
    cudaGraph_t g = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue_steps(s, GRAPH_STEPS);
    cudaError_t e = cudaStreamEndCapture(s->stream, &g);
    if (rc != NFX_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return fail(NFX_ERR_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&s->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(NFX_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    s->graph_valid = true;
    return NFX_OK;
}

// A new material: the captured graph holds the kernel of one material model, so it is rebuilt only
// when the model changes; parameters travel through the table.
void set_material(nfx_sim* s, const MaterialDev& m) {
    if (!s->have_material || s->cell.mat.model != m.model) invalidate_graph(s);
    s->cell.mat = m;
    s->cell_dirty = true;
    s->have_material = true;
}

void note_rows(nfx_sim* s, long long t_begin, long long t_end_inclusive) {
    // rows produced by node passes at times in [t_begin, t_end_inclusive]
    const long long every = s->record_every;
    if (s->cell.record_contact < 0 || every <= 0 || t_end_inclusive < t_begin) return;
    const long long last = t_end_inclusive / every;  // last row index touched
    if (last * every >= t_begin) s->rows_written = std::max(s->rows_written, std::min(last + 1, s->curve_rows));
}

// The per-node and per-tetra state a checkpoint holds, in the device's internal order: the
// displacement hi/lo, velocity and previous force of every node and, for the viscoplastic law,
// the plastic state and the stress fields of every tetra slot. The force accumulator is zero
// between steps (the node pass clears it) and is not part of the state.
struct StateArray {
    void* ptr;
    size_t bytes;
};
std::vector<StateArray> state_arrays(const nfx_sim* s) {
    const size_t np = (size_t)s->plan.np;
    std::vector<StateArray> a = {{s->st.ua, np * sizeof(float4)},
                                 {s->st.ub, np * sizeof(float2)},
                                 {s->st.va, np * sizeof(float4)},
                                 {s->st.vb, np * sizeof(float2)}};
    if (s->cell.mat.model == MODEL_VP && s->st.vp_a) {
        const size_t ntp = (size_t)s->plan.nslots + ARRAY_PAD;
        a.push_back({s->st.vp_a, ntp * sizeof(float4)});
        a.push_back({s->st.vp_b, ntp * sizeof(float4)});
        a.push_back({s->st.vp_c, ntp * sizeof(float2)});
        a.push_back({s->st.fields, ntp * sizeof(float2)});
    }
    return a;
}

constexpr uint64_t CKPT_MAGIC = 0x3130544b43584e46ull;  // "NFXCKT01" little-endian
struct CkptHeader {
    uint64_t magic;
    int64_t np, nt, nslots;
    int32_t tile_tets, model;
    int64_t time, rows;   // simulation time, force-curve rows stored after the state
    uint32_t status, n_arrays;
    uint64_t state_bytes;  // bytes of the state arrays (after the header)
};

int64_t checkpoint_bytes(const nfx_sim* s, int64_t* rows_out) {
    uint64_t b = sizeof(CkptHeader);
    for (const StateArray& a : state_arrays(s)) b += a.bytes;
    const int64_t rows = s->cell.record_contact >= 0 ? std::min<long long>(s->rows_written, s->curve_rows) : 0;
    if (rows_out) *rows_out = rows;
    return (int64_t)(b + 3 * sizeof(double) * (uint64_t)rows);
}

}  // namespace

extern "C" {

int nfx_version(void) { return 100; }

int nfx_plan_check(int64_t np, int64_t nt, const double* points, const uint32_t* tets, int tile_tets,
                   int64_t* ntiles, int64_t* node_entries) {
    CHECK_ARG(points && tets && ntiles && node_entries, "null argument");
    MeshPlan P;
    std::string err;
    if (!build_mesh_plan(np, nt, points, tets, tile_tets, P, err)) return fail(NFX_ERR_ARG, err);
    const int64_t T = P.tile_tets, NM = std::min<int64_t>(T, TILE_NODES_MAX);
    auto bad = [&](const std::string& what) { return fail(NFX_ERR_STATE, "plan_check: " + what); };
    if (P.nslots != P.ntiles * T || (int64_t)P.tile_meta.size() != P.ntiles) return bad("tile counts");
    std::vector<int> seen((size_t)nt, 0);
    int64_t entries = 0;
    for (int64_t b = 0; b < P.ntiles; b++) {
        const int64_t ntt = P.tile_meta[b] & 0xffffu, nn = P.tile_meta[b] >> 16;
        if (ntt < 1 || ntt > T || nn < 1 || nn > NM) return bad("tile " + std::to_string(b) + " sizes");
        entries += nn;
        std::vector<int> uses((size_t)nn, 0);
        for (int64_t j = 0; j < T; j++) {
            const int64_t slot = b * T + j, ut = P.tet_user[slot];
            if (j >= ntt) {
                if (ut != -1) return bad("padding slot holds a tetra");
                continue;
            }
            if (ut < 0 || ut >= nt || seen[ut]++) return bad("tetra missing or repeated");
            for (int k = 0; k < 4; k++) {
                const int64_t loc = P.lconn[4 * slot + k];
                if (loc >= nn) return bad("corner index past the tile's nodes");
                const uint32_t id = P.tile_nodes[2 * (b * NM + loc)];
                if (P.node_user[id] != (int64_t)tets[k * nt + ut]) return bad("corner names the wrong node");
                uses[loc]++;
            }
        }
        // incidence list: node q's run holds exactly its corners, as corner-major slots, in order
        uint32_t prev_count = 0xffffffffu;
        for (int64_t q = 0; q < nn; q++) {
            const uint32_t w = P.tile_nodes[2 * (b * NM + q) + 1], first = w >> 16, count = w & 0xffffu;
            if ((int)count != uses[q] || count > prev_count) return bad("incidence counts");
            prev_count = count;
            int last = -1;
            for (uint32_t e = 0; e < count; e++) {
                const uint32_t v = P.tile_inc[4 * b * T + first + e], k = v / T, j = v % T;
                if ((int64_t)j >= ntt || P.lconn[4 * (b * T + j) + k] != q) return bad("incidence entry");
                const int order = (int)(4 * j + k);
                if (order <= last) return bad("incidence order");
                last = order;
            }
        }
    }
    for (int64_t t = 0; t < nt; t++)
        if (seen[t] != 1) return bad("tetra not covered");
    // fixed-point range: every tile that lists a node adds at most fix_max * 2^40 units per
    // component to the node's signed 64-bit word, so (tiles per node) * fix_max * 2^40 < 2^63
    std::vector<int64_t> tiles_of((size_t)np, 0);
    for (int64_t b = 0; b < P.ntiles; b++)
        for (int64_t q = 0; q < (int64_t)(P.tile_meta[b] >> 16); q++) tiles_of[P.tile_nodes[2 * (b * NM + q)]]++;
    const int64_t busiest = *std::max_element(tiles_of.begin(), tiles_of.end());
    if (busiest != P.max_tiles_per_node) return bad("tiles per node");
    if (!((double)busiest * (double)P.fix_max * (double)FORCE_FIX_SCALE < 9223372036854775808.0))
        return bad("fixed-point bound can overflow a node's accumulator");
    *ntiles = P.ntiles;
    *node_entries = entries;
    return NFX_OK;
}

int nfx_last_error(char* buf, size_t len) {
    if (!buf || len == 0) return NFX_ERR_ARG;
    std::snprintf(buf, len, "%s", g_err.c_str());
    return NFX_OK;
}

int nfx_create(int device, nfx_sim** out) {
    if (!out) return fail(NFX_ERR_ARG, "out is null");
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0)
        return fail(NFX_ERR_NODEVICE, std::string("no CUDA device: ") + cudaGetErrorString(e));
    if (device < 0 || device >= count)
        return fail(NFX_ERR_NODEVICE, "device id " + std::to_string(device) + " does not exist (" +
                                           std::to_string(count) + " devices)");
    nfx_sim* s = new nfx_sim();
    s->device = device;
    int rc;
    if ((rc = set_device(s)) != NFX_OK) { delete s; return rc; }
    e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete s; return fail(NFX_ERR_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e)); }
    if ((rc = dalloc(s, &s->d_status, 1, nullptr)) != NFX_OK || (rc = dalloc(s, &s->d_clock, 1, nullptr)) != NFX_OK ||
        (rc = dalloc(s, &s->d_counter, 1, nullptr)) != NFX_OK || (rc = dalloc(s, &s->d_force_out, 1, nullptr)) != NFX_OK ||
        (rc = dalloc(s, &s->d_cell, 1, nullptr)) != NFX_OK) {
        nfx_destroy(s);
        return rc;
    }
    cudaMemsetAsync(s->d_status, 0, sizeof(unsigned), s->stream);
    cudaMemsetAsync(s->d_clock, 0, sizeof(StepClock), s->stream);
    cudaMemsetAsync(s->d_counter, 0, sizeof(unsigned), s->stream);
    s->st.status = s->d_status;
    s->st.clock = s->d_clock;
    s->st.force_out = s->d_force_out;
    s->cell.record_contact = -1;
    s->cell.fix_a = s->cell.fix_b = -1;
    s->cell.si_contact = -1;
    s->cell.integrator = INTEGRATOR_VV;
    if (const char* v = std::getenv("NFX_TILE_TETS")) {
        const int t = std::atoi(v);
        if (t == 64 || t == 128 || t == 256 || t == 512) s->tile_tets = t;
    }
    // default integrator: the reference's xi = 0.005 (VelocityVerlet.cl:11)
    const double xi = 0.005;
    s->cell.vv_a = (float)((1 - 0.5 * xi) / (1 + 0.5 * xi));
    s->cell.vv_hb = (float)(0.5 / (1 + 0.5 * xi));
    s->cell.vv_dm = (float)(1 - 0.5 * xi);
    *out = s;
    return NFX_OK;
}

int nfx_destroy(nfx_sim* s) {
    if (!s) return NFX_OK;
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    invalidate_graph(s);
    free_mesh(s);
    if (s->copy_stream) cudaStreamDestroy(s->copy_stream);
    if (s->ev_snap) cudaEventDestroy(s->ev_snap);
    if (s->ev_copy) cudaEventDestroy(s->ev_copy);
    for (int c = 0; c < MAX_CONTACTS; c++)
        for (int k = 0; k < 2; k++) {
            if (s->d_tables[c][k]) cudaFree(s->d_tables[c][k]);
            if (s->d_meta[c][k]) cudaFree(s->d_meta[c][k]);
            if (s->ev_table[c][k]) cudaEventDestroy(s->ev_table[c][k]);
        }
    if (s->d_curve) cudaFree(s->d_curve);
    if (s->d_status) cudaFree(s->d_status);
    if (s->d_clock) cudaFree(s->d_clock);
    if (s->d_counter) cudaFree(s->d_counter);
    if (s->d_force_out) cudaFree(s->d_force_out);
    if (s->d_cell) cudaFree(s->d_cell);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return NFX_OK;
}

int nfx_set_mesh(nfx_sim* s, int64_t np, int64_t nt, const double* points, const uint32_t* tets) {
    CHECK_ARG(s, "null handle");
    CHECK_ARG(points && tets, "null points or tets");
    int rc;
    if ((rc = set_device(s)) != NFX_OK) return rc;
    MeshPlan plan;
    std::string err;
    if (!build_mesh_plan(np, nt, points, tets, s->tile_tets, plan, err)) return fail(NFX_ERR_ARG, err);
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    invalidate_graph(s);
    free_mesh(s);
    s->plan = std::move(plan);
    const MeshPlan& P = s->plan;
    auto& A = s->mesh_allocs;
    int* tb; int* nbg; unsigned* tm; uint2* tn; uchar4* lc; ushort4* ti; float4 *da, *db; float2* dc;
    float4 *xh, *xl, *ua, *va, *bbox; float2 *ub, *vb; unsigned long long* fa; double* part; double* tpart;
    const size_t nblk = (size_t)((np + NODE_BLOCK - 1) / NODE_BLOCK);
    const int64_t ns = P.nslots;
    const size_t ntp = (size_t)ns + ARRAY_PAD;  // per-slot arrays carry ARRAY_PAD zeroed elements
    if ((rc = dalloc(s, &tb, P.tile_tet_begin.size(), &A)) || (rc = dalloc(s, &nbg, P.tile_node_begin.size(), &A)) ||
        (rc = dalloc(s, &tm, P.tile_meta.size(), &A)) ||
        (rc = dalloc(s, &tn, P.tile_nodes.size() / 2 + ARRAY_PAD, &A)) || (rc = dalloc(s, &lc, ntp, &A)) ||
        (rc = dalloc(s, &ti, ntp, &A)) ||
        (rc = dalloc(s, &da, ntp, &A)) || (rc = dalloc(s, &db, ntp, &A)) || (rc = dalloc(s, &dc, ntp, &A)) ||
        (rc = dalloc(s, &xh, (size_t)np, &A)) || (rc = dalloc(s, &xl, (size_t)np, &A)) || (rc = dalloc(s, &ua, (size_t)np, &A)) ||
        (rc = dalloc(s, &ub, (size_t)np, &A)) || (rc = dalloc(s, &va, (size_t)np, &A)) || (rc = dalloc(s, &vb, (size_t)np, &A)) ||
        (rc = dalloc(s, &fa, 3 * (size_t)np, &A)) || (rc = dalloc(s, &part, (size_t)((np + NODE_BLOCK - 1) / NODE_BLOCK), &A)) ||
        (rc = dalloc(s, &tpart, (size_t)P.ntiles, &A)) || (rc = dalloc(s, &bbox, 2 * nblk, &A)) ||
        (rc = dalloc(s, &s->d_node_user, (size_t)np, &A)) || (rc = dalloc(s, &s->d_stage, 9 * (size_t)std::max(np, ns), &A))) {
        free_mesh(s);
        return rc;
    }
    // per-tetra constants, split into the float4/float4/float2 streams the kernel reads
    std::vector<float> a(4 * (size_t)ns), b(4 * (size_t)ns), c(2 * (size_t)ns);
    for (int64_t t = 0; t < ns; t++) {
        const float* o = &P.dmi[12 * t];
        for (int k = 0; k < 4; k++) a[4 * t + k] = o[k];
        for (int k = 0; k < 4; k++) b[4 * t + k] = o[4 + k];
        c[2 * t] = o[8];
        c[2 * t + 1] = o[9];
    }
    std::vector<long long> nu(P.node_user.begin(), P.node_user.end());
    cudaStream_t st = s->stream;
    // zero the padding so bulk copies past a tile's end read defined values
    CUDA_TRY(cudaMemsetAsync(tn, 0, (P.tile_nodes.size() / 2 + ARRAY_PAD) * sizeof(uint2), st));
    CUDA_TRY(cudaMemsetAsync(lc, 0, ntp * sizeof(uchar4), st));
    CUDA_TRY(cudaMemsetAsync(ti, 0, ntp * sizeof(ushort4), st));
    CUDA_TRY(cudaMemsetAsync(da, 0, ntp * sizeof(float4), st));
    CUDA_TRY(cudaMemsetAsync(db, 0, ntp * sizeof(float4), st));
    CUDA_TRY(cudaMemsetAsync(dc, 0, ntp * sizeof(float2), st));
    CUDA_TRY(cudaMemcpyAsync(tb, P.tile_tet_begin.data(), P.tile_tet_begin.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(nbg, P.tile_node_begin.data(), P.tile_node_begin.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(tn, P.tile_nodes.data(), P.tile_nodes.size() * sizeof(unsigned), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(tm, P.tile_meta.data(), P.tile_meta.size() * sizeof(unsigned), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(lc, P.lconn.data(), P.lconn.size(), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(ti, P.tile_inc.data(), P.tile_inc.size() * sizeof(uint16_t), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(da, a.data(), a.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(db, b.data(), b.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(dc, c.data(), c.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(xh, P.Xh.data(), P.Xh.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(xl, P.Xl.data(), P.Xl.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(bbox, P.block_box.data(), P.block_box.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(s->d_node_user, nu.data(), nu.size() * sizeof(long long), cudaMemcpyHostToDevice, st));
    for (float4* z : {ua, va}) CUDA_TRY(cudaMemsetAsync(z, 0, (size_t)np * sizeof(float4), st));
    for (float2* z : {ub, vb}) CUDA_TRY(cudaMemsetAsync(z, 0, (size_t)np * sizeof(float2), st));
    CUDA_TRY(cudaMemsetAsync(fa, 0, 3 * (size_t)np * sizeof(unsigned long long), st));
    CUDA_TRY(cudaMemsetAsync(s->d_clock, 0, sizeof(StepClock), st));
    CUDA_TRY(launch_advance_time(s->st, 0, s->fields_every, s->record_every, st));
    CUDA_TRY(cudaMemsetAsync(s->d_status, 0, sizeof(unsigned), st));
    CUDA_TRY(cudaStreamSynchronize(st));  // host vectors a/b/c/nu go out of scope
    s->mesh.np = (int)np;
    s->mesh.nt = (int)nt;
    s->mesh.ntiles = (int)P.ntiles;
    s->mesh.tile_tets = P.tile_tets;
    s->mesh.tile_tet_begin = tb;
    s->mesh.tile_node_begin = nbg;
    s->mesh.tile_nodes = tn;
    s->mesh.tile_meta = tm;
    s->mesh.lconn = lc;
    s->mesh.tile_inc = ti;
    s->mesh.dmi_a = da;
    s->mesh.dmi_b = db;
    s->mesh.dmi_c = dc;
    s->mesh.Xh = xh;
    s->mesh.Xl = xl;
    s->mesh.fix_max = P.fix_max;
    s->mesh.block_box = bbox;
    s->st.ua = ua;
    s->st.ub = ub;
    s->st.va = va;
    s->st.vb = vb;
    s->st.facc = fa;
    s->st.partials = part;
    s->st.tile_partials = tpart;
    s->time = 0;
    s->rows_written = 0;
    s->nblocks = (int)((np + NODE_BLOCK - 1) / NODE_BLOCK);
    s->cell.fix_a = s->cell.fix_b = -1;
    s->cell.node_begin = 0;
    s->cell.node_end = (int)np;
    s->cell.block_begin = 0;
    s->cell.block_end = s->nblocks;
    s->cell.tile_begin = 0;
    s->cell.tile_end = (int)P.ntiles;
    s->cell_dirty = true;
    s->have_mesh = true;
    // the viscoplastic state follows the mesh
    if (s->have_material && s->cell.mat.model == MODEL_VP) {
        s->have_material = false;
        return fail(NFX_ERR_STATE, "mesh replaced: call nfx_set_viscoplastic again");
    }
    return NFX_OK;
}

int nfx_set_tetra(nfx_sim* s, int model, double E, double nu, double mr) {
    CHECK_ARG(s, "null handle");
    CHECK_ARG(model == NFX_MODEL_MR || model == NFX_MODEL_SVK || model == NFX_MODEL_SVKK, "unknown elastic model");
    CHECK_ARG(std::isfinite(E) && std::isfinite(nu) && std::isfinite(mr), "non-finite material parameter");
    CHECK_ARG(nu != 0.5, "poisson ratio 0.5 makes the bulk modulus infinite");
    // constants of tetra.cl:79-84, :97-102, :118-121
    const double mu = E / (2 * (1 + nu));
    MaterialDev m{};
    m.model = model;
    m.mu1 = (float)(mr * mu);
    m.mu2 = (float)((1 - mr) * mu);
    m.kappa = (float)(E / (3 * (1 - 2 * nu)));
    m.mu = (float)mu;
    m.kp = (float)(nu / (1 - 2 * nu));
    set_material(s, m);
    return NFX_OK;
}

int nfx_set_viscoplastic(nfx_sim* s, const double* par) {
    CHECK_ARG(s && par, "null argument");
    if (!s->have_mesh) return fail(NFX_ERR_STATE, "no mesh: call nfx_set_mesh first");
    for (int k = 0; k < 8; k++) CHECK_ARG(std::isfinite(par[k]), "non-finite viscoplastic parameter");
    CHECK_ARG(par[4] > 0, "yield stress must be positive");
    CHECK_ARG(par[6] != 0, "hardening threshold must be non-zero");
    int rc;
    if ((rc = set_device(s)) != NFX_OK) return rc;
    const size_t ntp = (size_t)s->plan.nslots + ARRAY_PAD;
    if (!s->st.vp_a) {
        if ((rc = dalloc(s, &s->st.vp_a, ntp, &s->mesh_allocs)) || (rc = dalloc(s, &s->st.vp_b, ntp, &s->mesh_allocs)) ||
            (rc = dalloc(s, &s->st.vp_c, ntp, &s->mesh_allocs)) || (rc = dalloc(s, &s->st.fields, ntp, &s->mesh_allocs)))
            return rc;
    }
    CUDA_TRY(cudaMemsetAsync(s->st.vp_a, 0, ntp * sizeof(float4), s->stream));
    CUDA_TRY(cudaMemsetAsync(s->st.vp_b, 0, ntp * sizeof(float4), s->stream));
    CUDA_TRY(cudaMemsetAsync(s->st.vp_c, 0, ntp * sizeof(float2), s->stream));
    CUDA_TRY(cudaMemsetAsync(s->st.fields, 0, ntp * sizeof(float2), s->stream));
    MaterialDev m{};
    m.model = MODEL_VP;
    m.mu1 = (float)par[0];
    m.mu2 = (float)par[1];
    m.kappa = (float)par[2];
    m.flow_exp = (float)par[3];
    m.yield = (float)par[4];
    m.flow_rate = (float)par[5];
    m.hard_thr = (float)par[6];
    m.hard_exp = (float)par[7];
    set_material(s, m);
    return NFX_OK;
}

int nfx_add_contact(nfx_sim* s, int kind, double k, double radius, double p0, double v, double tmove, int* id) {
    CHECK_ARG(s, "null handle");
    CHECK_ARG(kind == NFX_CONTACT_SUBSTRATE || kind == NFX_CONTACT_PLANE || kind == NFX_CONTACT_SPHERE ||
                  kind == NFX_CONTACT_SPHERE_INTEGRAL,
              "unknown contact kind");
    CHECK_ARG(s->cell.n_contacts < MAX_CONTACTS, "at most 4 contacts");
    CHECK_ARG(kind != NFX_CONTACT_SPHERE_INTEGRAL || s->cell.si_contact < 0, "at most one integrated sphere contact");
    CHECK_ARG(std::isfinite(k) && std::isfinite(p0) && std::isfinite(v) && !std::isnan(tmove), "non-finite contact parameter");
    CHECK_ARG((kind != NFX_CONTACT_SPHERE && kind != NFX_CONTACT_SPHERE_INTEGRAL) || radius > 0,
              "sphere radius must be positive");
    int rc;
    if ((rc = set_device(s)) != NFX_OK) return rc;
    const int i = s->cell.n_contacts;
    for (int k = 0; k < 2; k++) {
        if (!s->d_meta[i][k] && (rc = dalloc(s, &s->d_meta[i][k], 2, nullptr)) != NFX_OK) return rc;
        CUDA_TRY(cudaMemsetAsync(s->d_meta[i][k], 0, 2 * sizeof(long long), s->stream));
    }
    s->table_cur[i] = 0;
    ContactDev c{};
    c.kind = kind;
    c.k = k;
    c.radius = radius;
    c.p0 = p0;
    c.v = v;
    c.tmove = tmove;
    c.table = s->d_tables[i][0];
    c.meta = s->d_meta[i][0];
    s->cell.c[i] = c;
    s->cell.n_contacts++;
    if (kind == NFX_CONTACT_SPHERE_INTEGRAL) {
        s->cell.si_contact = i;
        invalidate_graph(s);  // the step gains the integrated sphere's pass
    }
    s->cell_dirty = true;
    if (id) *id = i;
    return NFX_OK;
}

int nfx_set_contact_table(nfx_sim* s, int id, int64_t t0, int64_t n, const double* pos) {
    CHECK_ARG(s, "null handle");
    CHECK_ARG(id >= 0 && id < s->cell.n_contacts, "contact id out of range");
    CHECK_ARG(n >= 0 && (n == 0 || pos), "bad table");
    for (int64_t k = 0; k < n; k++) CHECK_ARG(std::isfinite(pos[k]), "non-finite table position");
    int rc;
    if ((rc = set_device(s)) != NFX_OK) return rc;
    // fill the buffer the enqueued steps do not read, once the work that last read it is done
    const int cur = s->table_cur[id], nxt = 1 - cur;
    if (s->ev_table_set[id][nxt]) CUDA_TRY(cudaEventSynchronize(s->ev_table[id][nxt]));
    if (n > s->table_cap[id][nxt]) {
        if (s->d_tables[id][nxt]) cudaFree(s->d_tables[id][nxt]);
        s->d_tables[id][nxt] = nullptr;
        s->table_cap[id][nxt] = 0;
        const long long cap = std::max<long long>(n, 4096);
        if ((rc = dalloc(s, &s->d_tables[id][nxt], (size_t)cap, nullptr)) != NFX_OK) return rc;
        s->table_cap[id][nxt] = cap;
    }
    const long long meta[2] = {(long long)t0, (long long)n};
    // Copies from pageable memory have taken the bytes when they return and run in stream order;
    // the positions go through a pageable copy so that the caller may reuse its array at once even
    // when it is page-locked.
    if (n > 0) {
        const std::vector<double> staged(pos, pos + n);
        CUDA_TRY(cudaMemcpyAsync(s->d_tables[id][nxt], staged.data(), (size_t)n * sizeof(double),
                                 cudaMemcpyHostToDevice, s->stream));
    }
    CUDA_TRY(cudaMemcpyAsync(s->d_meta[id][nxt], meta, sizeof(meta), cudaMemcpyHostToDevice, s->stream));
    // later steps read the new buffer; everything enqueued so far may still read the old one
    if (!s->ev_table[id][cur]) CUDA_TRY(cudaEventCreateWithFlags(&s->ev_table[id][cur], cudaEventDisableTiming));
    CUDA_TRY(cudaEventRecord(s->ev_table[id][cur], s->stream));
    s->ev_table_set[id][cur] = true;
    s->cell.c[id].table = s->d_tables[id][nxt];
    s->cell.c[id].meta = s->d_meta[id][nxt];
    s->table_cur[id] = nxt;
    s->cell_dirty = true;
    return upload_cell(s);
}

int nfx_set_integrator(nfx_sim* s, double xi, int fix_top_bottom) {
    CHECK_ARG(s, "null handle");
    CHECK_ARG(std::isfinite(xi) && xi > -2.0, "bad damping");
    // v' = (v (1 - xi/2) + (f + fo)/2) / (1 + xi/2);  x' = x + v'(1 - xi/2) + f/2  (VelocityVerlet.cl:12-14)
    if (fix_top_bottom && !s->have_mesh) return fail(NFX_ERR_STATE, "set the mesh before pinning nodes 3 and 4");
    s->cell.integrator = INTEGRATOR_VV;
    s->cell.vv_a = (float)((1 - 0.5 * xi) / (1 + 0.5 * xi));
    s->cell.vv_hb = (float)(0.5 / (1 + 0.5 * xi));
    s->cell.vv_dm = (float)(1 - 0.5 * xi);
    s->cell.fix_a = s->cell.fix_b = -1;
    if (fix_top_bottom) {
        if (s->plan.np > 3) s->cell.fix_a = (int)s->plan.node_int[3];
        if (s->plan.np > 4) s->cell.fix_b = (int)s->plan.node_int[4];
    }
    s->cell_dirty = true;
    return NFX_OK;
}

int nfx_set_integrator_lumped(nfx_sim* s, double xi, double density) {
    CHECK_ARG(s, "null handle");
    CHECK_ARG(std::isfinite(xi) && xi > -2.0, "bad damping");
    CHECK_ARG(std::isfinite(density) && density > 0, "density must be positive");
    // velocityVerlet2.cl:9-13 with the lumped masses of SimulationLegacy.py:911-924
    s->cell.integrator = INTEGRATOR_VV2;
    s->cell.vv2_c = (float)(1.0 / (1.0 + 0.5 * xi));
    s->cell.vv2_xi = (float)xi;
    s->cell.inv_density = (float)(1.0 / density);
    s->cell.fix_a = s->cell.fix_b = -1;
    s->cell_dirty = true;
    return NFX_OK;
}

int nfx_set_record(nfx_sim* s, int contact, int64_t every, int64_t max_rows) {
    CHECK_ARG(s, "null handle");
    CHECK_ARG(contact >= -1 && contact < s->cell.n_contacts, "contact id out of range");
    CHECK_ARG(contact < 0 || (every > 0 && max_rows > 0), "every and max_rows must be positive");
    int rc;
    if ((rc = set_device(s)) != NFX_OK) return rc;
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    snapshot_drain(s);
    if (contact >= 0 && max_rows > s->curve_rows) {
        if (s->d_curve) cudaFree(s->d_curve);
        s->d_curve = nullptr;
        s->curve_rows = 0;
        if ((rc = dalloc(s, &s->d_curve, 3 * (size_t)max_rows, nullptr)) != NFX_OK) return rc;
        s->curve_rows = max_rows;
    }
    if (s->d_curve) CUDA_TRY(cudaMemsetAsync(s->d_curve, 0, 3 * (size_t)s->curve_rows * sizeof(double), s->stream));
    s->cell.record_contact = contact;
    s->cell_dirty = true;
    s->record_every = contact >= 0 ? every : 0;
    s->max_rows = contact >= 0 ? max_rows : 0;
    s->fields_every = every > 0 ? every : 0;
    s->rows_written = 0;
    invalidate_graph(s);  // record settings and the curve buffer are kernel arguments
    CUDA_TRY(launch_advance_time(s->st, 0, s->fields_every, s->record_every, s->stream));
    return NFX_OK;
}

int nfx_step(nfx_sim* s, int64_t nsteps) {
    const NvtxRange range("nfx_step");
    int rc;
    if ((rc = require_ready(s)) != NFX_OK) return rc;
    CHECK_ARG(nsteps >= 0, "negative step count");
    if ((rc = set_device(s)) != NFX_OK) return rc;
    if ((rc = upload_cell(s)) != NFX_OK) return rc;
    const long long t_begin = s->time;
    int64_t left = nsteps;
    while (left >= GRAPH_STEPS) {
        if (!s->graph_valid && (rc = build_graph(s)) != NFX_OK) return rc;
        CUDA_TRY(cudaGraphLaunch(s->graph, s->stream));
        left -= GRAPH_STEPS;
    }
    if (left > 0 && (rc = enqueue_steps(s, (int)left)) != NFX_OK) return rc;
    s->time += nsteps;
    if (nsteps > 0) note_rows(s, t_begin, s->time - 1);
    return NFX_OK;
}

int nfx_record_now(nfx_sim* s) {
    int rc;
    if ((rc = require_ready(s)) != NFX_OK) return rc;
    if ((rc = set_device(s)) != NFX_OK) return rc;
    if (s->cell.record_contact < 0) return NFX_OK;
    if ((rc = upload_cell(s)) != NFX_OK) return rc;
    CUDA_TRY(prepare_readout(s, s->cell.record_contact));
    CUDA_TRY(launch_nodes(s, 0, NODE_READOUT_ROW, -1));
    note_rows(s, s->time, s->time);
    return NFX_OK;
}

int nfx_host_alloc(size_t bytes, void** out) {
    CHECK_ARG(out, "null argument");
    *out = nullptr;
    CUDA_TRY(cudaMallocHost(out, std::max<size_t>(bytes, 1)));
    return NFX_OK;
}

int nfx_host_free(void* p) {
    if (p) CUDA_TRY(cudaFreeHost(p));
    return NFX_OK;
}

int nfx_sync(nfx_sim* s) {
    CHECK_ARG(s, "null handle");
    int rc;
    if ((rc = set_device(s)) != NFX_OK) return rc;
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    return NFX_OK;
}

int nfx_get_time(nfx_sim* s, int64_t* t) {
    CHECK_ARG(s && t, "null argument");
    *t = s->time;
    return NFX_OK;
}

int nfx_get_points(nfx_sim* s, double* out) {
    CHECK_ARG(s && out, "null argument");
    if (!s->have_mesh) return fail(NFX_ERR_STATE, "no mesh");
    int rc;
    if ((rc = set_device(s)) != NFX_OK) return rc;
    CUDA_TRY(launch_points_to_user(s->mesh, s->st, s->d_node_user, s->d_stage, s->stream));
    CUDA_TRY(cudaMemcpyAsync(out, s->d_stage, 3 * (size_t)s->plan.np * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    return NFX_OK;
}

int nfx_set_points(nfx_sim* s, const double* in) {
    CHECK_ARG(s && in, "null argument");
    if (!s->have_mesh) return fail(NFX_ERR_STATE, "no mesh");
    int rc;
    if ((rc = set_device(s)) != NFX_OK) return rc;
    CUDA_TRY(cudaMemcpyAsync(s->d_stage, in, 3 * (size_t)s->plan.np * sizeof(double), cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(launch_points_from_user(s->mesh, s->st, s->d_node_user, s->d_stage, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    return NFX_OK;
}

// part 0: the velocity, part 1: the previous force (va/vb)
static int get_vec(nfx_sim* s, int part, double* out) {
    CHECK_ARG(s && out, "null argument");
    if (!s->have_mesh) return fail(NFX_ERR_STATE, "no mesh");
    int rc;
    if ((rc = set_device(s)) != NFX_OK) return rc;
    CUDA_TRY(launch_vec_to_user(s->mesh, s->st.va, s->st.vb, part, s->d_node_user, s->d_stage, s->stream));
    CUDA_TRY(cudaMemcpyAsync(out, s->d_stage, 3 * (size_t)s->plan.np * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    return NFX_OK;
}

static int set_vec(nfx_sim* s, int part, const double* in) {
    CHECK_ARG(s && in, "null argument");
    if (!s->have_mesh) return fail(NFX_ERR_STATE, "no mesh");
    int rc;
    if ((rc = set_device(s)) != NFX_OK) return rc;
    CUDA_TRY(cudaMemcpyAsync(s->d_stage, in, 3 * (size_t)s->plan.np * sizeof(double), cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(launch_vec_from_user(s->mesh, s->st.va, s->st.vb, part, s->d_node_user, s->d_stage, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    return NFX_OK;
}

int nfx_get_velocities(nfx_sim* s, double* out) { return s ? get_vec(s, 0, out) : fail(NFX_ERR_ARG, "null handle"); }
int nfx_set_velocities(nfx_sim* s, const double* in) { return s ? set_vec(s, 0, in) : fail(NFX_ERR_ARG, "null handle"); }
int nfx_get_force_old(nfx_sim* s, double* out) { return s ? get_vec(s, 1, out) : fail(NFX_ERR_ARG, "null handle"); }
int nfx_set_force_old(nfx_sim* s, const double* in) { return s ? set_vec(s, 1, in) : fail(NFX_ERR_ARG, "null handle"); }

int nfx_get_tet_field(nfx_sim* s, int which, double* out) {
    CHECK_ARG(s && out, "null argument");
    CHECK_ARG(which >= 0 && which <= 2, "unknown field");
    if (!s->have_mesh) return fail(NFX_ERR_STATE, "no mesh");
    const int64_t nt = s->plan.nt, ns = s->plan.nslots;
    if (s->cell.mat.model != MODEL_VP || !s->st.vp_c) {
        // the elastic kernel (tetra.cl) writes no per-tetra fields; the reference's buffers stay 0
        std::fill(out, out + nt, 0.0);
        return NFX_OK;
    }
    int rc;
    if ((rc = set_device(s)) != NFX_OK) return rc;
    std::vector<float> h(2 * (size_t)ns);
    const float2* src = which == 2 ? s->st.vp_c : s->st.fields;
    CUDA_TRY(cudaMemcpyAsync(h.data(), src, (size_t)ns * sizeof(float2), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    const int comp = which == 0 ? 0 : 1;
    for (int64_t t = 0; t < ns; t++)
        if (s->plan.tet_user[t] >= 0) out[s->plan.tet_user[t]] = (double)h[2 * t + comp];
    return NFX_OK;
}

int nfx_get_plastic_tensor(nfx_sim* s, double* out) {
    CHECK_ARG(s && out, "null argument");
    if (!s->have_mesh) return fail(NFX_ERR_STATE, "no mesh");
    const int64_t nt = s->plan.nt;
    if (s->cell.mat.model != MODEL_VP || !s->st.vp_a) {
        for (int k = 0; k < 9; k++)
            for (int64_t t = 0; t < nt; t++) out[k * nt + t] = (k % 4 == 0) ? 1.0 : 0.0;
        return NFX_OK;
    }
    int rc;
    if ((rc = set_device(s)) != NFX_OK) return rc;
    const int64_t ns = s->plan.nslots;
    std::vector<float> a(4 * (size_t)ns), b(4 * (size_t)ns), c(2 * (size_t)ns);
    CUDA_TRY(cudaMemcpyAsync(a.data(), s->st.vp_a, (size_t)ns * sizeof(float4), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaMemcpyAsync(b.data(), s->st.vp_b, (size_t)ns * sizeof(float4), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaMemcpyAsync(c.data(), s->st.vp_c, (size_t)ns * sizeof(float2), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    for (int64_t t = 0; t < ns; t++) {
        const int64_t u = s->plan.tet_user[t];
        if (u < 0) continue;  // padding slot
        const float P[9] = {a[4 * t], a[4 * t + 1], a[4 * t + 2], a[4 * t + 3], b[4 * t], b[4 * t + 1],
                            b[4 * t + 2], b[4 * t + 3], c[2 * t]};
        for (int k = 0; k < 9; k++) out[k * nt + u] = (double)P[k] + ((k % 4 == 0) ? 1.0 : 0.0);
    }
    return NFX_OK;
}

int nfx_get_curve(nfx_sim* s, double* rows, int64_t max_rows, int64_t* n_rows) {
    CHECK_ARG(s && n_rows, "null argument");
    CHECK_ARG(max_rows >= 0 && (max_rows == 0 || rows), "bad row buffer");
    int rc;
    if ((rc = set_device(s)) != NFX_OK) return rc;
    const long long n = std::min<long long>(s->rows_written, max_rows);
    if (n > 0) {
        CUDA_TRY(cudaMemcpyAsync(rows, s->d_curve, 3 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    }
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    *n_rows = s->rows_written;
    return NFX_OK;
}

int nfx_snapshot(nfx_sim* s, double* points_out, double* rows_out, int64_t max_rows, int64_t* n_rows) {
    CHECK_ARG(s && points_out && n_rows, "null argument");
    CHECK_ARG(max_rows >= 0 && (max_rows == 0 || rows_out), "bad row buffer");
    if (!s->have_mesh) return fail(NFX_ERR_STATE, "no mesh");
    int rc;
    if ((rc = set_device(s)) != NFX_OK) return rc;
    if (!s->copy_stream) {
        CUDA_TRY(cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking));
        CUDA_TRY(cudaEventCreateWithFlags(&s->ev_snap, cudaEventDisableTiming));
        CUDA_TRY(cudaEventCreateWithFlags(&s->ev_copy, cudaEventDisableTiming));
    }
    const size_t bytes = 3 * (size_t)s->plan.np * sizeof(double);
    if (!s->d_snap && (rc = dalloc(s, &s->d_snap, 3 * (size_t)s->plan.np, nullptr)) != NFX_OK) return rc;
    // the previous snapshot's copy must have left the staging buffer before it is rewritten
    if (s->snap_pending) CUDA_TRY(cudaStreamWaitEvent(s->stream, s->ev_copy, 0));
    CUDA_TRY(launch_points_to_user(s->mesh, s->st, s->d_node_user, s->d_snap, s->stream));
    CUDA_TRY(cudaEventRecord(s->ev_snap, s->stream));
    CUDA_TRY(cudaStreamWaitEvent(s->copy_stream, s->ev_snap, 0));
    CUDA_TRY(cudaMemcpyAsync(points_out, s->d_snap, bytes, cudaMemcpyDeviceToHost, s->copy_stream));
    // rows already recorded are final: later steps only write rows after them
    const long long n = std::min<long long>(s->rows_written, max_rows);
    if (n > 0)
        CUDA_TRY(cudaMemcpyAsync(rows_out, s->d_curve, 3 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost,
                                 s->copy_stream));
    CUDA_TRY(cudaEventRecord(s->ev_copy, s->copy_stream));
    s->snap_pending = true;
    *n_rows = s->rows_written;
    return NFX_OK;
}

int nfx_snapshot_wait(nfx_sim* s) {
    CHECK_ARG(s, "null handle");
    int rc;
    if ((rc = set_device(s)) != NFX_OK) return rc;
    if (!s->snap_pending) return NFX_OK;
    const cudaError_t e = cudaEventSynchronize(s->ev_copy);
    s->snap_pending = false;
    if (e != cudaSuccess) return fail(NFX_ERR_CUDA, std::string("snapshot: ") + cudaGetErrorString(e));
    return NFX_OK;
}

int nfx_indenter_force(nfx_sim* s, int contact, double* out) {
    int rc;
    if ((rc = require_ready(s)) != NFX_OK) return rc;
    CHECK_ARG(out, "null out");
    CHECK_ARG(contact >= 0 && contact < s->cell.n_contacts, "contact id out of range");
    if ((rc = set_device(s)) != NFX_OK) return rc;
    if ((rc = upload_cell(s)) != NFX_OK) return rc;
    CUDA_TRY(prepare_readout(s, contact));
    CUDA_TRY(launch_nodes(s, 0, NODE_READOUT_VALUE, contact));
    CUDA_TRY(cudaMemcpyAsync(out, s->d_force_out, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    return NFX_OK;
}

int nfx_status(nfx_sim* s, uint32_t* flags, int clear) {
    CHECK_ARG(s && flags, "null argument");
    int rc;
    if ((rc = set_device(s)) != NFX_OK) return rc;
    unsigned h = 0;
    CUDA_TRY(cudaMemcpyAsync(&h, s->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, s->stream));
    if (clear) CUDA_TRY(cudaMemsetAsync(s->d_status, 0, sizeof(unsigned), s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    *flags = h;
    return NFX_OK;
}

int nfx_time_steps(nfx_sim* s, int64_t nsteps, float* ms) {
    CHECK_ARG(s && ms, "null argument");
    int rc;
    if ((rc = require_ready(s)) != NFX_OK) return rc;
    if ((rc = set_device(s)) != NFX_OK) return rc;
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    CUDA_TRY(cudaEventRecord(e0, s->stream));
    rc = nfx_step(s, nsteps);
    cudaEventRecord(e1, s->stream);
    cudaError_t e = cudaEventSynchronize(e1);
    float t = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != NFX_OK) return rc;
    if (e != cudaSuccess) return fail(NFX_ERR_CUDA, std::string("event timing: ") + cudaGetErrorString(e));
    *ms = t;
    return NFX_OK;
}

int nfx_profile_steps(nfx_sim* s, int64_t nsteps, float* tet_ms, float* node_ms) {
    CHECK_ARG(s && tet_ms && node_ms, "null argument");
    CHECK_ARG(nsteps >= 0 && nsteps <= (1 << 20), "bad step count");
    int rc;
    if ((rc = require_ready(s)) != NFX_OK) return rc;
    if ((rc = set_device(s)) != NFX_OK) return rc;
    if ((rc = upload_cell(s)) != NFX_OK) return rc;
    std::vector<cudaEvent_t> ev(3 * (size_t)nsteps + 1);
    for (auto& e : ev) CUDA_TRY(cudaEventCreate(&e));
    const long long t_begin = s->time;
    cudaError_t err = cudaSuccess;
    // one step per clock advance, so the step offset stays inside the clock's window
    for (int64_t k = 0; k < nsteps && err == cudaSuccess; k++) {
        cudaEventRecord(ev[3 * k], s->stream);
        err = launch_elem(s, 0);
        if (err == cudaSuccess) err = launch_si(s, 0);
        cudaEventRecord(ev[3 * k + 1], s->stream);
        if (err == cudaSuccess) err = launch_nodes(s, 0, NODE_UPDATE, -1);
        cudaEventRecord(ev[3 * k + 2], s->stream);
        if (err == cudaSuccess) err = launch_advance_time(s->st, 1, s->fields_every, s->record_every, s->stream);
    }
    if (err == cudaSuccess) err = cudaStreamSynchronize(s->stream);
    float a = 0.f, b = 0.f;
    for (int64_t k = 0; k < nsteps && err == cudaSuccess; k++) {
        float x = 0.f, y = 0.f;
        err = cudaEventElapsedTime(&x, ev[3 * k], ev[3 * k + 1]);
        if (err == cudaSuccess) err = cudaEventElapsedTime(&y, ev[3 * k + 1], ev[3 * k + 2]);
        a += x;
        b += y;
    }
    for (auto& e : ev) cudaEventDestroy(e);
    if (err != cudaSuccess) return fail(NFX_ERR_CUDA, std::string("profile_steps: ") + cudaGetErrorString(err));
    s->time += nsteps;
    if (nsteps > 0) note_rows(s, t_begin, s->time - 1);
    *tet_ms = a;
    *node_ms = b;
    return NFX_OK;
}

int nfx_profile_tet_pass(nfx_sim* s, int launches, float* ms) {
    CHECK_ARG(s && ms, "null argument");
    CHECK_ARG(launches >= 1 && launches <= 4096, "launch count out of range [1, 4096]");
    int rc;
    if ((rc = require_ready(s)) != NFX_OK) return rc;
    if ((rc = set_device(s)) != NFX_OK) return rc;
    if ((rc = upload_cell(s)) != NFX_OK) return rc;
    // The element pass advances the plastic state (and may write the stress fields): keep a copy
    // of both and put it back afterwards.
    const bool vp = s->cell.mat.model == MODEL_VP && s->st.vp_a;
    const size_t ntp = (size_t)s->plan.nslots + ARRAY_PAD;
    std::vector<void*> keep;
    auto release = [&]() {
        for (void* q : keep) cudaFree(q);
    };
    if (vp) {
        const void* src[4] = {s->st.vp_a, s->st.vp_b, s->st.vp_c, s->st.fields};
        const size_t bytes[4] = {ntp * sizeof(float4), ntp * sizeof(float4), ntp * sizeof(float2), ntp * sizeof(float2)};
        for (int i = 0; i < 4; i++) {
            void* q = nullptr;
            cudaError_t e = cudaMalloc(&q, bytes[i]);
            if (e != cudaSuccess) {
                release();
                return fail(NFX_ERR_NOMEM, std::string("profile_tet_pass: cudaMalloc: ") + cudaGetErrorString(e));
            }
            keep.push_back(q);
            e = cudaMemcpyAsync(q, src[i], bytes[i], cudaMemcpyDeviceToDevice, s->stream);
            if (e != cudaSuccess) {
                release();
                return fail(NFX_ERR_CUDA, std::string("profile_tet_pass: save: ") + cudaGetErrorString(e));
            }
        }
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t err = cudaEventCreate(&e0);
    if (err == cudaSuccess) err = cudaEventCreate(&e1);
    if (err == cudaSuccess) err = cudaEventRecord(e0, s->stream);
    for (int k = 0; k < launches && err == cudaSuccess; k++) err = launch_elem(s, 0);
    if (err == cudaSuccess) err = cudaEventRecord(e1, s->stream);
    float t = 0.f;
    if (err == cudaSuccess) err = cudaEventSynchronize(e1);
    if (err == cudaSuccess) err = cudaEventElapsedTime(&t, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    // Undo the passes' effects: the accumulated forces and, for the viscoplastic law, the state.
    if (err == cudaSuccess)
        err = cudaMemsetAsync(s->st.facc, 0, 3 * (size_t)s->mesh.np * sizeof(unsigned long long), s->stream);
    if (vp && err == cudaSuccess) {
        void* dst[4] = {s->st.vp_a, s->st.vp_b, s->st.vp_c, s->st.fields};
        const size_t bytes[4] = {ntp * sizeof(float4), ntp * sizeof(float4), ntp * sizeof(float2), ntp * sizeof(float2)};
        for (int i = 0; i < 4 && err == cudaSuccess; i++)
            err = cudaMemcpyAsync(dst[i], keep[i], bytes[i], cudaMemcpyDeviceToDevice, s->stream);
    }
    if (err == cudaSuccess) err = cudaStreamSynchronize(s->stream);
    release();
    if (err != cudaSuccess) return fail(NFX_ERR_CUDA, std::string("profile_tet_pass: ") + cudaGetErrorString(err));
    *ms = t / (float)launches;
    return NFX_OK;
}

int nfx_divide_check(int device, int64_t n, const float* a, const float* b, float* q) {
    CHECK_ARG(a && b && q, "null argument");
    CHECK_ARG(n >= 0 && n <= (int64_t)1 << 26, "n out of range [0, 2^26]");
    if (n == 0) return NFX_OK;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return fail(NFX_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    float* d = nullptr;
    const size_t bytes = (size_t)n * sizeof(float);
    e = cudaMalloc(&d, 3 * bytes);
    if (e != cudaSuccess) return fail(NFX_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    e = cudaMemcpy(d, a, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d + n, b, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = launch_divide_check(d, d + n, d + 2 * n, (long long)n, 0);
    if (e == cudaSuccess) e = cudaMemcpy(q, d + 2 * n, bytes, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return fail(NFX_ERR_CUDA, std::string("divide_check: ") + cudaGetErrorString(e));
    return NFX_OK;
}

int nfx_checkpoint_size(nfx_sim* s, int64_t* bytes) {
    int rc;
    if ((rc = require_ready(s)) != NFX_OK) return rc;
    CHECK_ARG(bytes, "null argument");
    *bytes = checkpoint_bytes(s, nullptr);
    return NFX_OK;
}

int nfx_checkpoint_save(nfx_sim* s, void* buf, int64_t bytes) {
    int rc;
    if ((rc = require_ready(s)) != NFX_OK) return rc;
    CHECK_ARG(buf, "null buffer");
    int64_t rows = 0;
    const int64_t need = checkpoint_bytes(s, &rows);
    CHECK_ARG(bytes >= need, "checkpoint buffer too small: " + std::to_string((long long)need) + " bytes needed");
    if ((rc = set_device(s)) != NFX_OK) return rc;
    CUDA_TRY(cudaStreamSynchronize(s->stream));  // every enqueued step has finished
    snapshot_drain(s);
    const std::vector<StateArray> arrays = state_arrays(s);
    CkptHeader h{};
    h.magic = CKPT_MAGIC;
    h.np = s->plan.np;
    h.nt = s->plan.nt;
    h.nslots = s->plan.nslots;
    h.tile_tets = s->plan.tile_tets;
    h.model = s->cell.mat.model;
    h.time = s->time;
    h.rows = rows;
    h.n_arrays = (uint32_t)arrays.size();
    unsigned status = 0;
    CUDA_TRY(cudaMemcpyAsync(&status, s->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, s->stream));
    char* p = static_cast<char*>(buf) + sizeof(CkptHeader);
    for (const StateArray& a : arrays) {
        CUDA_TRY(cudaMemcpyAsync(p, a.ptr, a.bytes, cudaMemcpyDeviceToHost, s->stream));
        p += a.bytes;
        h.state_bytes += a.bytes;
    }
    if (rows > 0) CUDA_TRY(cudaMemcpyAsync(p, s->d_curve, 3 * sizeof(double) * (size_t)rows, cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    h.status = status;
    std::memcpy(buf, &h, sizeof(h));
    return NFX_OK;
}

int nfx_checkpoint_load(nfx_sim* s, const void* buf, int64_t bytes) {
    int rc;
    if ((rc = require_ready(s)) != NFX_OK) return rc;
    CHECK_ARG(buf && bytes >= (int64_t)sizeof(CkptHeader), "checkpoint buffer too small");
    CkptHeader h;
    std::memcpy(&h, buf, sizeof(h));
    CHECK_ARG(h.magic == CKPT_MAGIC, "not a checkpoint of this library");
    CHECK_ARG(h.np == s->plan.np && h.nt == s->plan.nt && h.nslots == s->plan.nslots &&
                  h.tile_tets == s->plan.tile_tets,
              "checkpoint of a different mesh or tile size");
    CHECK_ARG(h.model == s->cell.mat.model, "checkpoint of a different material model");
    const std::vector<StateArray> arrays = state_arrays(s);
    uint64_t state_bytes = 0;
    for (const StateArray& a : arrays) state_bytes += a.bytes;
    CHECK_ARG(h.n_arrays == arrays.size() && h.state_bytes == state_bytes, "checkpoint state layout differs");
    CHECK_ARG(h.rows >= 0 && (uint64_t)bytes >= sizeof(CkptHeader) + state_bytes + 3 * sizeof(double) * (uint64_t)h.rows,
              "checkpoint truncated");
    CHECK_ARG(h.rows == 0 || (s->cell.record_contact >= 0 && h.rows <= s->curve_rows),
              "the checkpoint holds force rows: call nfx_set_record with at least as many rows first");
    CHECK_ARG(h.time >= 0, "negative checkpoint time");
    if ((rc = set_device(s)) != NFX_OK) return rc;
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    snapshot_drain(s);
    const char* p = static_cast<const char*>(buf) + sizeof(CkptHeader);
    for (const StateArray& a : arrays) {
        CUDA_TRY(cudaMemcpyAsync(a.ptr, p, a.bytes, cudaMemcpyHostToDevice, s->stream));
        p += a.bytes;
    }
    if (h.rows > 0) CUDA_TRY(cudaMemcpyAsync(s->d_curve, p, 3 * sizeof(double) * (size_t)h.rows, cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(cudaMemsetAsync(s->st.facc, 0, 3 * (size_t)s->plan.np * sizeof(unsigned long long), s->stream));
    CUDA_TRY(cudaMemcpyAsync(s->d_status, &h.status, sizeof(unsigned), cudaMemcpyHostToDevice, s->stream));
    const long long t = h.time;
    CUDA_TRY(cudaMemcpyAsync(&s->d_clock->time, &t, sizeof(long long), cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(launch_advance_time(s->st, 0, s->fields_every, s->record_every, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    s->time = t;
    s->rows_written = h.rows;
    return NFX_OK;
}

int nfx_set_plastic_tensor(nfx_sim* s, const double* in) {
    CHECK_ARG(s && in, "null argument");
    if (!s->have_mesh) return fail(NFX_ERR_STATE, "no mesh");
    if (s->cell.mat.model != MODEL_VP || !s->st.vp_a)
        return fail(NFX_ERR_STATE, "no viscoplastic material: call nfx_set_viscoplastic first");
    const int64_t nt = s->plan.nt, ns = s->plan.nslots;
    for (int64_t i = 0; i < 9 * nt; i++) CHECK_ARG(std::isfinite(in[i]), "non-finite plastic tensor entry");
    int rc;
    if ((rc = set_device(s)) != NFX_OK) return rc;
    // keep the accumulated strain, replace P = Fp - I
    std::vector<float> a(4 * (size_t)ns, 0.f), b(4 * (size_t)ns, 0.f), c(2 * (size_t)ns, 0.f);
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    CUDA_TRY(cudaMemcpyAsync(c.data(), s->st.vp_c, (size_t)ns * sizeof(float2), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    for (int64_t t = 0; t < ns; t++) {
        const int64_t u = s->plan.tet_user[t];
        if (u < 0) continue;
        float P[9];
        for (int k = 0; k < 9; k++) P[k] = (float)(in[k * nt + u] - ((k % 4 == 0) ? 1.0 : 0.0));
        for (int k = 0; k < 4; k++) a[4 * t + k] = P[k];
        for (int k = 0; k < 4; k++) b[4 * t + k] = P[4 + k];
        c[2 * t] = P[8];
    }
    CUDA_TRY(cudaMemcpyAsync(s->st.vp_a, a.data(), (size_t)ns * sizeof(float4), cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(cudaMemcpyAsync(s->st.vp_b, b.data(), (size_t)ns * sizeof(float4), cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(cudaMemcpyAsync(s->st.vp_c, c.data(), (size_t)ns * sizeof(float2), cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));  // the host vectors go out of scope
    return NFX_OK;
}

int nfx_mesh_info(nfx_sim* s, int64_t* ntiles, int64_t* tile_nodes) {
    CHECK_ARG(s && ntiles && tile_nodes, "null argument");
    if (!s->have_mesh) return fail(NFX_ERR_STATE, "no mesh");
    *ntiles = s->plan.ntiles;
    int64_t nodes = 0;
    for (uint32_t m : s->plan.tile_meta) nodes += m >> 16;
    *tile_nodes = nodes;
    return NFX_OK;
}

}  // extern "C"
