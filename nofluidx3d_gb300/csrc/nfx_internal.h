// Internal data structures shared by the host runtime (nfx_api.cpp, nfx_mesh.cpp) and the
// kernels (nfx_kernels.cu). Not part of the C ABI.
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstdint>
#include <string>
#include <vector>

namespace nfx {

enum Model : int { MODEL_MR = 0, MODEL_SVK = 1, MODEL_SVKK = 2, MODEL_VP = 3 };
enum ContactKind : int { CONTACT_SUBSTRATE = 0, CONTACT_PLANE = 1, CONTACT_SPHERE = 2, CONTACT_SPHERE_INTEGRAL = 3 };
enum Integrator : int { INTEGRATOR_VV = 0, INTEGRATOR_VV2 = 1 };

constexpr int MAX_CONTACTS = 4;
// A tile is a run of consecutive tetrahedra (after reordering) processed by one CTA. Its
// distinct nodes are listed once, so the per-tetra connectivity is four 8-bit local indices
// and the tile's nodal forces are summed in shared memory before one flush per node.
constexpr int DEFAULT_TILE_TETS = 128;  // fastest measured on GB300 (R=64 viscoplastic cell)
constexpr int TILE_NODES_MAX = 256;  // 8-bit local corner indices
// Tile sizes the one-CTA-per-tile kernel is built for; a tile has at most min(tile, 256) nodes.
constexpr int TILE_SIZES[4] = {64, 128, 256, 512};
constexpr int NODE_BLOCK = 256;

// Fixed-point scale of the force accumulator: 2^40 (resolution 9.1e-13, range +-8.4e6).
constexpr float FORCE_FIX_SCALE = 1099511627776.0f;
constexpr float FORCE_FIX_INV = 1.0f / 1099511627776.0f;
// A node's accumulator word receives one fixed-point tile sum from every tile that lists the
// node, so the per-tile bound is the word's range (2^63 units = 8,388,608 force units) shared
// out over the most tiles any node of the mesh appears in: FORCE_FIX_BUDGET / max tiles (never
// above FORCE_FIX_MAX). A tile sum above the bound raises STATUS_NONFINITE instead of being
// added, so no sum of in-bound tile sums can wrap the 64-bit word.
constexpr float FORCE_FIX_BUDGET = 8.0e6f;
constexpr float FORCE_FIX_MAX = 4.0e6f;
// The per-tile bound of a mesh whose busiest node appears in max_tiles tiles.
inline float force_fix_bound(int max_tiles) {
    const float b = FORCE_FIX_BUDGET / (float)(max_tiles > 0 ? max_tiles : 1);
    return b < FORCE_FIX_MAX ? b : FORCE_FIX_MAX;
}

// Status bits raised by the kernels (read back by nfx_status).
constexpr unsigned STATUS_NONFINITE = 1u;   // a position or force became NaN/Inf
constexpr unsigned STATUS_INVERTED = 2u;    // an element reached det F <= 0
constexpr unsigned STATUS_CURVE_FULL = 4u;  // a record row fell outside the curve buffer
constexpr unsigned STATUS_TIMEOUT = 8u;     // reserved: a bounded device wait gave up (no current kernel waits)

// Extra zeroed elements after every per-tetra array and the tile node list (slack for loads
// that run past a tile's last real element).
constexpr int ARRAY_PAD = 16;

// ---------------------------------------------------------------------------------------
// Host-side mesh plan: reordering, tiles, per-tetra reference quantities.
// ---------------------------------------------------------------------------------------
// Tiles sit at a fixed stride: tile b owns tetra slots [b*T, (b+1)*T) and node-list entries
// [b*NMAX, (b+1)*NMAX), NMAX = min(T, 256); slots and entries past the tile's real counts
// (tile_meta) are zero padding.
struct MeshPlan {
    int64_t np = 0, nt = 0, ntiles = 0;
    int64_t nslots = 0;                    // ntiles * tile_tets
    int tile_tets = DEFAULT_TILE_TETS;
    std::vector<int64_t> node_user;   // internal node -> user node id
    std::vector<int64_t> node_int;    // user node id -> internal node
    std::vector<int64_t> tet_user;    // tetra slot -> user tetra id, -1 for padding
    std::vector<int32_t> tile_tet_begin;   // ntiles + 1 (= b*T)
    std::vector<int32_t> tile_node_begin;  // ntiles + 1 (= b*NMAX)
    std::vector<uint32_t> tile_meta;       // per tile: tetra count | node count << 16
    std::vector<uint32_t> tile_nodes;      // 2 per node entry: internal node id, (first << 16 | count)
                                           // of its run in the tile's incidence list
    std::vector<uint8_t> lconn;            // 4 * nslots local corner indices
    std::vector<uint16_t> tile_inc;        // 4 * nslots: per tile, the corners (corner * tile size + local tet)
                                           // grouped by local node in node order, tet order within
    std::vector<float> dmi;                // 12 * nslots: Dm^-1 row-major (9), V0, pad, pad
    std::vector<float> Xh, Xl;             // 4 * np: reference position hi / lo parts; Xh.w holds the
                                           // inverse lumped mass of density 1 (VelocityVerlet2)
    std::vector<float> block_box;          // 8 per node block of NODE_BLOCK internal nodes: bounding box
                                           // of the reference positions (lo xyz, 0, hi xyz, 0), outward-rounded
    int max_tiles_per_node = 1;            // the most tiles that list any one node
    float fix_max = FORCE_FIX_MAX;         // per-tile fixed-point bound, force_fix_bound(max_tiles_per_node)
};

// Builds the plan from the reference's layouts (points SoA 3*np doubles, tets SoA 4*nt).
// Returns false with a message on invalid input (index out of range, degenerate tetra).
bool build_mesh_plan(int64_t np, int64_t nt, const double* points_soa, const uint32_t* tets_soa, int tile_tets,
                     MeshPlan& plan, std::string& err);

// ---------------------------------------------------------------------------------------
// Device views passed to kernels by value.
// ---------------------------------------------------------------------------------------
struct MeshDev {
    int np, nt, ntiles;
    int tile_tets;
    const int* tile_tet_begin;
    const int* tile_node_begin;
    const unsigned* tile_meta; // tetra count | node count << 16
    const uint2* tile_nodes;   // (node id, first << 16 | count)
    const uchar4* lconn;
    const ushort4* tile_inc;   // four incidence entries per tetra slot of the tile
    const float4* dmi_a;  // Dm^-1 entries 0..3
    const float4* dmi_b;  // Dm^-1 entries 4..7
    const float2* dmi_c;  // Dm^-1 entry 8, V0
    const float4* Xh;  // w: inverse lumped mass at density 1
    const float4* Xl;
    const float4* block_box;  // per node block: (lo x, y, z, -), (hi x, y, z, -) of the reference
                              // positions, rounded outwards
    float fix_max;     // per-tile fixed-point bound of the accumulator (force_fix_bound)
    int tile_base;     // index of this launch's first tile in the batch-wide tile numbering
                       // (tile_partials, CellDev::tile_begin/tile_end); 0 for a single cell
};

// Device-side step clock: the simulation time at the start of the current chunk of launches and,
// for the next CLOCK_WINDOW steps (t_offset 0 .. CLOCK_WINDOW-1), bitmasks of the steps that
// write the per-tetra fields and of those that record a curve row. k_advance_time refreshes the
// masks whenever it moves the time, so a step tests one bit instead of dividing 64-bit integers
// on every thread. Every chunk of launches between two refreshes stays within the window.
constexpr int CLOCK_WINDOW = 128;
struct StepClock {
    long long time;
    unsigned fields_due[CLOCK_WINDOW / 32];  // bit k: (time + k + 1) % fields_every == 0
    unsigned record_due[CLOCK_WINDOW / 32];  // bit k: (time + k) % record_every == 0
};

// Node state, 48 bytes per node with no padding lane: the displacement u = x - X as float
// hi + lo parts (ua: hi x, y, z and lo x; ub: lo y, z) and the velocity and previous force (va:
// v x, y, z and f_old x; vb: f_old y, z). The element pass gathers ua/ub (24 B per tile node), the
// node pass streams all four; the float4 + float2 split keeps every access a 16- or 8-byte
// vector load at its natural alignment.
struct StateDev {
    float4* ua;     // displacement hi (x, y, z), displacement lo x
    float2* ub;     // displacement lo (y, z)
    float4* va;     // velocity (x, y, z), previous force x (previous acceleration: lumped-mass integrator)
    float2* vb;     // previous force (y, z)
    // Element-force accumulator, 3 * np signed 64-bit fixed-point values (component d of node
    // i at [d*np + i], FORCE_FIX_SCALE units per force unit), zeroed by the node pass. Integer
    // addition is associative, so the sum does not depend on the order of the atomics.
    unsigned long long* facc;
    float4* vp_a;   // viscoplastic P = Fp - I, entries 0..3
    float4* vp_b;   // entries 4..7
    float2* vp_c;   // entry 8, accumulated plastic strain
    float2* fields; // von Mises, pressure per tetra (viscoplastic model)
    unsigned* status;
    StepClock* clock;    // time at the start of the current chunk + schedule masks
    double* partials;    // one per node block, for the deterministic readout reduction
    double* tile_partials;  // one per tile: the tile's share of an integrated-sphere readout
    double* force_out;   // per cell: result of an on-demand readout
};

struct ContactDev {
    int kind;
    int pad;
    double k, radius;
    double p0, v, tmove;
    // Optional per-step positions in device memory: meta = {t0, n}; n = 0 means "use the
    // schedule". Kept in memory (not in the kernel parameters) so a captured graph stays
    // valid when the host refills the table.
    const double* table;
    const long long* meta;
};

struct MaterialDev {
    int model;
    float mu1, mu2, kappa;  // Mooney-Rivlin / Neo-Hookean (and the viscoplastic elastic law)
    float mu, kp;           // SVK / SVKK: mu and nu/(1-2nu)
    float flow_exp, yield, flow_rate, hard_thr, hard_exp;
};

// ---------------------------------------------------------------------------------------
// Per-cell parameters. The kernels read every material, contact and integrator parameter from
// a device table of cells, never from kernel arguments: a single simulation is a table of one
// cell, a batch concatenates many cells' tile/tetra/node arrays and maps each tile and each node
// block to its cell. Both therefore run the same kernels with the same arithmetic, and a
// captured CUDA graph stays valid when the host rewrites a parameter in the table.
// Each cell's nodes occupy whole node blocks, so a node block belongs to exactly one cell.
// ---------------------------------------------------------------------------------------
struct CellDev {
    MaterialDev mat;
    int n_contacts;
    ContactDev c[MAX_CONTACTS];
    float vv_a, vv_hb, vv_dm;
    int fix_a, fix_b;             // global node ids of the pinned nodes, -1 if none
    int record_contact;           // -1: none
    int node_begin, node_end;     // the cell's nodes in the global arrays
    int block_begin, block_end;   // the cell's node blocks
    int tile_begin, tile_end;     // the cell's tiles
    int integrator;               // INTEGRATOR_VV (unit mass) or INTEGRATOR_VV2 (lumped masses)
    float vv2_c, vv2_xi, inv_density;  // VelocityVerlet2: 1 / (1 + xi/2), xi, 1 / density
    int si_contact;               // index of the integrated sphere contact, -1: none
};

struct BatchDev {
    const CellDev* cells;
    const int* tile_cell;        // per tile; null: every tile belongs to cell 0
    const int* block_cell;       // per node block; null: every block belongs to cell 0
    unsigned* cell_counter;      // per cell: blocks finished in the readout reduction
    unsigned* cell_status;       // per cell: status bits of that cell (null for a single simulation)
    double* curves;              // per cell: max_rows rows of (t, indentation, force)
    long long record_every;      // 0: no force recording
    long long max_rows;
    long long fields_every;      // tet fields written when (t+1) % fields_every == 0
};

// An NVTX range for the lifetime of the object (a step block, a batch step, a training run), so
// that a profiler's timeline shows the library's work by call; without an attached tool the
// NVTX calls return at once.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// Sets the message nfx_last_error() returns on this thread (nfx_api.cpp).
void set_error(const std::string& msg);

// Kernel launchers (nfx_kernels.cu). All enqueue on `stream` and return cudaGetLastError().
// Element pass over all tiles (one CTA per tile), material from the cell table. pdl: as a
// programmatic dependent launch (the kernel waits before any read, so after any predecessor).
cudaError_t launch_tet_pass(const MeshDev& m, const StateDev& s, const BatchDev& b, int model, int t_offset,
                            cudaStream_t stream, bool pdl = false);
enum NodeMode : int { NODE_UPDATE = 0, NODE_READOUT_ROW = 1, NODE_READOUT_VALUE = 2 };
// Node pass over `nblocks` node blocks. NODE_READOUT_VALUE sums contact `readout_contact`'s force
// per cell into force_out[cell] without updating the state.
// pdl: programmatic dependent launch, for the NODE_UPDATE pass of a run of steps only (its
// predecessor then is an element or integrated-sphere pass, launched in plain stream order).
cudaError_t launch_node_pass(const MeshDev& m, const StateDev& s, const BatchDev& b, int nblocks, int t_offset,
                             int mode, int readout_contact, cudaStream_t stream, bool pdl = false);
// Advance the clock by n steps (n = 0: refresh the masks only) for the given schedules.
cudaError_t launch_advance_time(const StateDev& s, long long n, long long fields_every, long long record_every,
                                cudaStream_t stream);
// Integrated sphere contact over all tiles (tiles of cells without one return at once). Inside a
// step (readout false): its forces join the accumulator and, on record steps, the tile partials
// of the readout are written. readout true: only the tile partials of contact index `contact` at
// the current positions, for readouts between steps.
cudaError_t launch_si_pass(const MeshDev& m, const StateDev& s, const BatchDev& b, int t_offset, bool readout,
                           int contact, cudaStream_t stream);
// q[i] = a[i] / b[i] with the element laws' device divide (self-check of its accuracy).
cudaError_t launch_divide_check(const float* a, const float* b, float* q, long long n, cudaStream_t stream);
// Conversions between the user's layout (SoA doubles, user order) and the device state.
cudaError_t launch_points_to_user(const MeshDev& m, const StateDev& s, const long long* node_user, double* out,
                                  cudaStream_t stream);
cudaError_t launch_points_from_user(const MeshDev& m, const StateDev& s, const long long* node_user,
                                    const double* in, cudaStream_t stream);
// A node vector stored split over a float4 and a float2 array: part 0 is (a.x, a.y, a.z), part 1
// is (a.w, b.x, b.y) — the velocity and the previous force of va/vb.
cudaError_t launch_vec_to_user(const MeshDev& m, const float4* a, const float2* b, int part, const long long* node_user,
                               double* out, cudaStream_t stream);
cudaError_t launch_vec_from_user(const MeshDev& m, float4* a, float2* b, int part, const long long* node_user,
                                 const double* in, cudaStream_t stream);
cudaError_t launch_init_vp(const MeshDev& m, const StateDev& s, cudaStream_t stream);

}  // namespace nfx
