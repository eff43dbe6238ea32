/*
 * nfx.h — C ABI of the GB300 implementation of noFluidX3D's explicit tetra-mesh time step.
 *
 * One nfx_sim handle is one cell simulation on one GPU: it owns the device buffers the
 * reference's Simulation and its Interaction plugins own (nofluidx3d/Simulation.py:82-90,
 * createBuffers of the plugins in nofluidx3d/interactions/) and runs the whole step — element forces, node
 * force accumulation, contacts, velocity Verlet, indenter-force readout — as CUDA kernels.
 *
 * Layout conventions are the reference's, so its Bridge host arrays (nofluidx3d/util/Bridge.py:16-26)
 * can be passed as they are:
 *   points / velocities / forces : double[3*np], SoA: x0..x_{np-1}, y0.., z0.. (Simulation.py:82-84)
 *   tetras                       : uint32[4*nt], SoA: corner k of tetra t at [k*nt + t] (Simulation.py:85-87)
 *   per-tetra fields             : double[nt]
 * Internally nodes and tetrahedra are reordered for locality; every getter/setter converts.
 *
 * All functions return NFX_OK (0) or an NFX_ERR_* code; nfx_last_error() gives the message of
 * the last failure on the calling thread. A handle must not be used from two threads at once.
 * Steps are enqueued asynchronously on the handle's CUDA stream; getters synchronise.
 */
#ifndef NFX_H
#define NFX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NFX_OK 0
#define NFX_ERR_ARG 1       /* invalid argument (null pointer, size, index out of range, degenerate mesh) */
#define NFX_ERR_CUDA 2      /* a CUDA runtime call failed (message has the CUDA error string) */
#define NFX_ERR_STATE 3     /* call out of order, e.g. nfx_step before nfx_set_mesh */
#define NFX_ERR_NOMEM 4     /* device allocation failed */
#define NFX_ERR_NODEVICE 5  /* no CUDA device with the requested index */

/* material models of nofluidx3d/interactions/Tetra.py:25-33 plus the viscoplastic law of
 * nofluidx3d/kernels/InteractionFiniteStrainViscoplastic.cl */
#define NFX_MODEL_MR 0   /* Mooney-Rivlin; Neo-Hookean is mooneyRivlinRatio = 1 (Tetra.py:77-78) */
#define NFX_MODEL_SVK 1  /* Saint-Venant-Kirchhoff (tetra.cl:94-114) */
#define NFX_MODEL_SVKK 2 /* Saint-Venant-Kirchhoff-Kellnberger (tetra.cl:76-93) */
#define NFX_MODEL_VP 3   /* finite-strain viscoplastic (InteractionFiniteStrainViscoplastic.cl:1-220) */

#define NFX_CONTACT_SUBSTRATE 0 /* nofluidx3d/interactions/Substrate.py, kernels/Interactions/Substrate.cl */
#define NFX_CONTACT_PLANE 1     /* nofluidx3d/interactions/Plane.py, kernels/Interactions/Plane.cl */
#define NFX_CONTACT_SPHERE 2    /* nofluidx3d/interactions/Sphere.py, kernels/Interactions/Sphere.cl */
#define NFX_CONTACT_SPHERE_INTEGRAL 3 /* Interactions.py:601-637, kernels/InteractionSphereIntegral.cl:22-85 */

/* status bits (nfx_status) */
#define NFX_STATUS_NONFINITE 1u  /* a position/velocity/force became NaN or Inf (util/IO.py:17-28 aborts on this) */
#define NFX_STATUS_INVERTED 2u   /* an element reached det F <= 0 */
#define NFX_STATUS_CURVE_FULL 4u /* a force-curve row fell outside the buffer given to nfx_set_record */
#define NFX_STATUS_TIMEOUT 8u    /* reserved: a bounded device wait gave up (the step is invalid); no current kernel waits */

/* per-tetra fields (nfx_get_tet_field) */
#define NFX_FIELD_VON_MISES 0   /* vonMises buffer, Simulation.py:89 */
#define NFX_FIELD_PRESSURE 1    /* pressure buffer, Simulation.py:90 (trace(sigma)/3, as the kernel writes it) */
#define NFX_FIELD_PLASTIC_STRAIN 2 /* accumulatedStrain, Interactions.py:276 */

typedef struct nfx_sim nfx_sim;

/* Library version, e.g. 100 for 0.1.0. */
int nfx_version(void);

/* Builds the device layout plan of a mesh on the host (no GPU needed) and checks its invariants:
 * every tetra in exactly one tile slot, tile sizes within bounds, corners naming the right
 * nodes, each node's incidence run holding exactly its corners in (tetra, corner) order, runs
 * ordered by decreasing length. Returns the tile count and the number of node entries over all
 * tiles. A planner self-check with no counterpart in the reference. */
int nfx_plan_check(int64_t np, int64_t nt, const double* points, const uint32_t* tets, int tile_tets,
                   int64_t* ntiles, int64_t* node_entries);

/* Copies the last error message of this thread into buf (NUL-terminated, truncated to len).
 * Replaces the reference's print()+exit() error paths (openCL.py:30-32, util/IO.py:17-28). */
int nfx_last_error(char* buf, size_t len);

/* Creates a simulation on CUDA device `device`. Replaces initializeOpenCLObjects(gpu)
 * (nofluidx3d/openCL.py:17-34): flat device index, one in-order stream. */
int nfx_create(int device, nfx_sim** out);

/* Frees all device and host resources of the handle. */
int nfx_destroy(nfx_sim* sim);

/* Uploads the cell mesh and resets the state (zero velocity, previous force and plastic state;
 * time 0). Replaces the shared Bridges points/tetras of Simulation.__init__ (Simulation.py:65-90)
 * plus the per-tetra reference quantities of Tetra.createBuffers (interactions/Tetra.py:49-64,
 * TetraCell.py:33-41), which are computed here once. points: double[3*np] SoA (reference
 * positions); tets: uint32[4*nt] SoA, positively oriented as tetra.cl:132 requires. */
int nfx_set_mesh(nfx_sim* sim, int64_t np, int64_t nt, const double* points, const uint32_t* tets);

/* Selects the elastic law with the reference's parameters: Tetra(cell, youngsModulus,
 * poissonRatio, mooneyRivlinRatio, model) (interactions/Tetra.py:35-47; constants of
 * tetra.cl:118-121). model: NFX_MODEL_MR / SVK / SVKK. */
int nfx_set_tetra(nfx_sim* sim, int model, double youngs_modulus, double poisson_ratio, double mooney_rivlin_ratio);

/* Selects the finite-strain viscoplastic law with uniform parameters
 * par = {mu1, mu2, kappa, flowExponent, yieldStress, plasticFlowRate, hardeningThreshhold,
 * hardeningExponent}: the constructor arguments of InteractionFiniteStrainViscoplastic
 * (nofluidx3d/Interactions.py:257-277). Resets the plastic state to Fp = I, strain 0. */
int nfx_set_viscoplastic(nfx_sim* sim, const double* par8);

/* Adds a contact interaction; *id receives its index (0..3), which is also its order of
 * application after the element force. position(t) = p0 - v*t while t <= tmove, then
 * p0 - v*tmove (the wallFunc/sphereFunc schedules of Simulation.py:117-132, :173-183);
 * substrate: position = p0. k is def_FORCE_CONST (Simulation.py:109, :134, :185).
 * Replaces Substrate(wallPosition, k), Plane(wallFunc, k), Sphere(radius, sphereFunc, k).
 * NFX_CONTACT_SPHERE_INTEGRAL replaces InteractionSphereIntegral(radius, sphereFunc, forceConst)
 * (SimulationLegacy.py:206-238): k is its PotentialForceConst (the decay rate of the density),
 * the force acts per tetra; at most one per simulation. */
int nfx_add_contact(nfx_sim* sim, int kind, double k, double radius, double p0, double v, double tmove, int* id);

/* Supplies explicit per-step positions pos[0..n) for times t0..t0+n-1 of contact `id`,
 * overriding its schedule; times outside the table use the nearest entry. This keeps
 * arbitrary host callables working: the reference re-evaluates wallFunc(t) on the host every
 * step in beforeTimeStep (interactions/Plane.py:39-41, Sphere.py:41-43). n = 0 removes it.
 * Stream-ordered: steps enqueued before the call use the previous table, later ones this one;
 * the call does not wait for the enqueued steps, and pos may be reused when it returns. */
int nfx_set_contact_table(nfx_sim* sim, int id, int64_t t0, int64_t n, const double* pos);

/* Velocity Verlet settings: damping xi (VelocityVerlet.cl:11 hard-codes 0.005) and the
 * FIXED_TOP_BOTTOM pin of user nodes 3 and 4 (VelocityVerlet.cl:17-22,
 * interactions/VelocityVerlet.py:23-45). */
int nfx_set_integrator(nfx_sim* sim, double xi, int fix_top_bottom);
/* The lumped-mass velocity Verlet instead (velocityVerlet2.cl:1-26, Interactions.py:818-836): nodal
 * masses density * sum of V0/4 over the node's tetrahedra (SimulationLegacy.py:911-924, where the
 * density is 1), damping xi, the old-force slot holding the previous acceleration. */
int nfx_set_integrator_lumped(nfx_sim* sim, double xi, double density);

/* Records the indenter force of contact `contact` every `every` steps into a device buffer of
 * max_rows rows (t, indentation, force) — the recordedQuantities currentTime / indentationSI /
 * forceSI of Simulation.py:94-100, :142-157, :194-216 in lattice units. Row r is time r*every.
 * Per-tetra fields (von Mises, pressure) are written by the step whose end time is a multiple of
 * `every`, as the reference's buffers hold the last step's values at each output
 * (util/IO.py:30-35). contact = -1 records no force rows but keeps the field interval. */
int nfx_set_record(nfx_sim* sim, int contact, int64_t every, int64_t max_rows);

/* Enqueues nsteps time steps (Simulation.timeStep, Simulation.py:232-237, nsteps times). */
int nfx_step(nfx_sim* sim, int64_t nsteps);

/* Computes the record row for the current time (when it is a record time) without stepping:
 * the readout the reference makes after the last step of a run (Simulation.py:274-278). */
int nfx_record_now(nfx_sim* sim);

/* Output snapshot without draining the step stream, for callers that write frames while the
 * simulation continues. Enqueues, after the steps enqueued so far, the node positions (user
 * order, SoA, as nfx_get_points) into `points_out` and the force rows recorded so far (up to
 * max_rows, as nfx_get_curve) into `rows_out`; returns at once with the number of recorded rows
 * in *n_rows. The host copies run on a second stream while later steps run; the buffers are
 * written asynchronously (page-locked host memory keeps the copies asynchronous) and may be read
 * only after nfx_snapshot_wait. A new snapshot may be taken before waiting for the previous one
 * (its device staging waits for the previous copy); nfx_snapshot_wait waits for the latest. The
 * reference reads positions synchronously at every output (util/IO.py:15); this is the
 * overlapped form of that readback. */
int nfx_snapshot(nfx_sim* sim, double* points_out, double* rows_out, int64_t max_rows, int64_t* n_rows);
int nfx_snapshot_wait(nfx_sim* sim);

/* Page-locked host memory (cudaMallocHost) for nfx_snapshot's buffers, so that callers without
 * a CUDA runtime of their own can overlap output copies with the steps; freed by nfx_host_free.
 * No counterpart in the reference. */
int nfx_host_alloc(size_t bytes, void** out);
int nfx_host_free(void* p);

/* Waits for all enqueued work of the handle. */
int nfx_sync(nfx_sim* sim);

/* Current simulation time in steps (Simulation.time). */
int nfx_get_time(nfx_sim* sim, int64_t* t);

/* Node positions x = X + u, double[3*np] SoA in user order (Bridge.readFromGPU of points,
 * util/IO.py:15). */
int nfx_get_points(nfx_sim* sim, double* out);

/* Overwrites node positions (Bridge.writeToGPU, util/Bridge.py:25-26). */
int nfx_set_points(nfx_sim* sim, const double* in);

/* Velocities, double[3*np] SoA (VelocityVerlet.velocityB, interactions/VelocityVerlet.py:29-33). */
int nfx_get_velocities(nfx_sim* sim, double* out);
int nfx_set_velocities(nfx_sim* sim, const double* in);

/* Total force of the last step, double[3*np] SoA (VelocityVerlet.forceOldB). */
int nfx_get_force_old(nfx_sim* sim, double* out);
int nfx_set_force_old(nfx_sim* sim, const double* in);

/* Per-tetra field in user tetra order (NFX_FIELD_*), double[nt]. */
int nfx_get_tet_field(nfx_sim* sim, int which, double* out);

/* Plastic deformation tensor Fp, double[9*nt] SoA (plasticDeformationTensor layout,
 * Interactions.py:279-281). */
int nfx_get_plastic_tensor(nfx_sim* sim, double* out);

/* Overwrites the plastic deformation tensor Fp, double[9*nt] SoA in user tetra order (the
 * plasticDeformationTensor buffer of Interactions.py:279-281 written back with writeToGPU); the
 * accumulated plastic strain is kept. Viscoplastic material only. */
int nfx_set_plastic_tensor(nfx_sim* sim, const double* in);

/* Checkpoint of the whole simulation state, for resuming a run bit for bit: node displacements
 * (hi and lo parts), velocities and previous forces, the viscoplastic state and stress fields,
 * the time, the status word and the force rows recorded so far, in the library's internal
 * order and precision. The reference's only restart reloads positions from a VTK frame
 * (SimulationLegacy.py:103-112, initCheckPointVTK), which loses velocities, forces and plastic
 * state. nfx_checkpoint_size gives the bytes nfx_checkpoint_save writes into a host buffer
 * (it waits for the enqueued steps first). nfx_checkpoint_load restores them into a handle set
 * up the same way (same mesh, material model and, when rows were saved, nfx_set_record with at
 * least as many rows); parameters, contacts and host position tables are set-up, not state, and
 * are not stored. */
int nfx_checkpoint_size(nfx_sim* sim, int64_t* bytes);
int nfx_checkpoint_save(nfx_sim* sim, void* buf, int64_t bytes);
int nfx_checkpoint_load(nfx_sim* sim, const void* buf, int64_t bytes);

/* Copies the recorded rows (3 doubles each) into rows; *n_rows receives how many rows exist
 * up to the current time (at most max_rows). */
int nfx_get_curve(nfx_sim* sim, double* rows, int64_t max_rows, int64_t* n_rows);

/* Indenter force of contact `contact` at the current time and positions, in lattice units:
 * the forceSI closures (Simulation.py:146-153 plane, :198-212 sphere) without p0*L0^2. */
int nfx_indenter_force(nfx_sim* sim, int contact, double* out);

/* Device status bits (NFX_STATUS_*), accumulated since the last call with clear != 0. */
int nfx_status(nfx_sim* sim, uint32_t* flags, int clear);

/* Enqueues nsteps steps like nfx_step, bracketed by CUDA events recorded on the handle's
 * stream, waits, and returns the elapsed device time in *ms. The reference only prints a
 * wall-clock steps/s figure (Simulation.py:281-286). */
int nfx_time_steps(nfx_sim* sim, int64_t nsteps, float* ms);

/* Runs nsteps steps launch by launch with CUDA events around every kernel and returns the
 * summed device time of the element passes (*tet_ms) and node passes (*node_ms). */
int nfx_profile_steps(nfx_sim* sim, int64_t nsteps, float* tet_ms, float* node_ms);

/* Average device time of one element pass (*ms), from `launches` back-to-back launches of the
 * pass for the current step between two CUDA events on the handle's stream. The passes' effects
 * (accumulated forces and, for the viscoplastic law, the plastic state and stress fields) are
 * undone before return. A timing helper with no counterpart in the reference. */
int nfx_profile_tet_pass(nfx_sim* sim, int launches, float* ms);

/* q[i] = a[i] / b[i] (host arrays of n floats) computed on `device` with the divide the element
 * laws use, so a test can check its accuracy against correctly rounded division. A self-check
 * with no counterpart in the reference. */
int nfx_divide_check(int device, int64_t n, const float* a, const float* b, float* q);

/* Number of mesh tiles and distinct-node entries (diagnostics for the tile layout). */
int nfx_mesh_info(nfx_sim* sim, int64_t* ntiles, int64_t* tile_nodes);

/* ------------------------------------------------------------------------------------------
 * Batched cells. The reference advances one cell per Simulation (nofluidx3d/Simulation.py:35);
 * a batch advances many independent cells of uneven size and material together: one element-pass
 * launch per size bucket and one node-pass launch per step for all cells, captured as a CUDA graph. All cells of
 * a batch use one material model; each has its own parameters, contacts, integrator settings and
 * force curve. Set-up calls come before nfx_batch_finalize; stepping and readback after.
 * ------------------------------------------------------------------------------------------ */
typedef struct nfx_batch nfx_batch;

/* tile_tets: 64, 128, 256 or 512 tetrahedra per tile for every cell, or 0 to group the cells by
 * size into buckets and let nfx_batch_finalize choose each bucket's tile size, timing a
 * representative sub-batch of the bucket with 64, 128 and 256 and keeping the fastest. */
int nfx_batch_create(int device, int tile_tets, nfx_batch** out);
int nfx_batch_destroy(nfx_batch* batch);
/* Adds a cell (layouts as nfx_set_mesh); *cell receives its index. */
int nfx_batch_add_cell(nfx_batch* batch, int64_t np, int64_t nt, const double* points, const uint32_t* tets, int* cell);
/* Adds a cell with the same mesh as cell `src` (no copy of the arrays; the plan is built once
 * for all cells sharing a mesh). Material, contacts and integrator are set per cell as usual. */
int nfx_batch_add_cell_like(nfx_batch* batch, int src, int* cell);
/* Per-cell material, as nfx_set_tetra / nfx_set_viscoplastic. */
int nfx_batch_set_tetra(nfx_batch* batch, int cell, int model, double youngs_modulus, double poisson_ratio,
                        double mooney_rivlin_ratio);
int nfx_batch_set_viscoplastic(nfx_batch* batch, int cell, const double* par8);
/* Per-cell contact (schedule only), as nfx_add_contact. */
int nfx_batch_add_contact(nfx_batch* batch, int cell, int kind, double k, double radius, double p0, double v,
                          double tmove, int* id);
/* Per-cell integrator, as nfx_set_integrator / nfx_set_integrator_lumped. */
int nfx_batch_set_integrator(nfx_batch* batch, int cell, double xi, int fix_top_bottom);
int nfx_batch_set_integrator_lumped(nfx_batch* batch, int cell, double xi, double density);
/* Records contact index `contact` of every cell every `every` steps into max_rows rows per cell. */
int nfx_batch_set_record(nfx_batch* batch, int contact, int64_t every, int64_t max_rows);
/* Builds the cells' plans on host threads (after autotuning the tile size when requested),
 * uploads them and zeroes the state. */
int nfx_batch_finalize(nfx_batch* batch);
/* Enqueues nsteps steps of every cell. */
int nfx_batch_step(nfx_batch* batch, int64_t nsteps);
/* nfx_batch_step bracketed by CUDA events on the batch's stream; waits; *ms = device time. */
int nfx_batch_time_steps(nfx_batch* batch, int64_t nsteps, float* ms);
/* Records the row of the current time for every cell (see nfx_record_now). */
int nfx_batch_record_now(nfx_batch* batch);
/* On-demand indenter force of contact index `contact` of every cell (Simulation.py:142-157,
 * evaluated per cell), out = double[cells]; a cell with fewer contacts reads 0. */
int nfx_batch_indenter_force(nfx_batch* batch, int contact, double* out);
/* Force curve of one cell (rows of t, indentation, force); *n_rows = rows available. */
int nfx_batch_get_curve(nfx_batch* batch, int cell, double* rows, int64_t max_rows, int64_t* n_rows);
/* Node positions of one cell, double[3*np] SoA in the cell's user order. */
int nfx_batch_get_points(nfx_batch* batch, int cell, double* out);
/* Overwrites the node positions of one cell (as nfx_set_points; Bridge.writeToGPU). */
int nfx_batch_set_points(nfx_batch* batch, int cell, const double* in);
int nfx_batch_status(nfx_batch* batch, uint32_t* flags, int clear);
/* The status bits of every cell, flags[cells] (the batch status is their union). */
int nfx_batch_cell_status(nfx_batch* batch, uint32_t* flags, int clear);
/* Cells, total tetrahedra and nodes, tile size in use. */
int nfx_batch_info(nfx_batch* batch, int64_t* cells, int64_t* tets, int64_t* nodes, int* tile_tets);
/* The autotuner's candidates and their times (ms for 10 steps of the sub-batch), bucket after
 * bucket (three candidates per bucket). */
int nfx_batch_tuning(nfx_batch* batch, int* tiles, float* ms, int max_n, int* n);
/* The buckets of a finalized batch: cells are grouped by size (up to 32,768 tetra, up to 262,144,
 * larger) when the tile size is autotuned, each bucket with its own tile size and its own
 * element-pass launch; a fixed tile size gives one bucket. Per bucket: tile size, cells, tetra. */
int nfx_batch_buckets(nfx_batch* batch, int max_n, int* n, int* tile_tets, int64_t* cells, int64_t* tets);

/* Indenter force of one contact on node positions the caller keeps in device memory, written
 * to one double in device memory. This entry point has no counterpart in the reference.
 *
 * It is for callers that cannot allocate device memory: a host solver that reserves its whole
 * device budget in its own pool at start-up and forbids any later cudaMalloc, or a coupling
 * loop that must not allocate (nor wait for the device synchronisation an allocation may bring)
 * between time steps. It allocates nothing. The per-block partial sums and the completion
 * counter of its fixed-order reduction live in one static device array of 128 KiB, which every
 * GPU that loads this library holds until the process exits; np is therefore limited to
 * NFX_NOALLOC_MAX_NODES, and a larger np returns NFX_ERR_ARG.
 *
 * Each call made outside stream capture looks up the array's device address in the current
 * context of `device` (so a reset device or another context gets its own copy); a call inside
 * a capture uses the address of the last uncaptured call, so make the first call on a device
 * before any stream capture. The call makes `device` current while it runs and restores the
 * caller's current device before it returns. Every call shares the array, and it keeps
 * the last call's contents (the counter is cleared at the start of each call): calls whose
 * work overlaps on the GPU — on different streams with no ordering between them — race and
 * give wrong results.
 *
 * points_dev: double[3*np] SoA in device memory; kind/k/radius as nfx_add_contact; position:
 * the contact's current position (plane/substrate height, sphere centre y); out_dev: one double
 * in device memory; stream: a cudaStream_t (NULL = the legacy default stream). Same contact laws
 * and sign as nfx_indenter_force. Errors are reported through nfx_last_error. */
#define NFX_NOALLOC_MAX_NODES 4194304
int nfx_indenter_force_noalloc(int device, int64_t np, const double* points_dev, int kind, double k, double radius,
                               double position, double* out_dev, void* stream);

/* ------------------------------------------------------------------------------------------
 * Surrogate MLP of the force-indentation curve. No counterpart in the reference (which has no
 * learned part): material parameters -> curve samples, n_in -> width (x depth hidden layers,
 * SiLU) -> n_out, BF16 weights and activations, FP32 accumulation (tensor-core MMAs), FP32
 * master weights and AdamW. Arrays are host pointers, row-major, FP32.
 * Parameter layout (nfx_mlp_set_params/get_params/get_grads): for each layer l in order,
 * W_l [out_l x in_l] row-major, then b_l [out_l].
 * ------------------------------------------------------------------------------------------ */
typedef struct nfx_mlp nfx_mlp;
/* n_in 1..16; width a multiple of 16 up to 1024; depth 1..7 hidden layers; n_out a multiple of
 * 8 up to 1024; max_batch rows per call. Parameters start at zero: set them before use. */
int nfx_mlp_create(int device, int n_in, int width, int depth, int n_out, int64_t max_batch, nfx_mlp** out);
int nfx_mlp_destroy(nfx_mlp* mlp);
int nfx_mlp_num_params(nfx_mlp* mlp, int64_t* n);
/* Output gain: y = exp(alpha * x[input]) * (last layer's output); input -1 removes it. The
 * gradients (parameters and inputs) are those of y. */
int nfx_mlp_set_output_gain(nfx_mlp* mlp, int input, float alpha);
/* Sets the FP32 master parameters (and their BF16 copies); resets the AdamW moments and step. */
int nfx_mlp_set_params(nfx_mlp* mlp, const float* params);
int nfx_mlp_get_params(nfx_mlp* mlp, float* params);
/* Gradients of the last nfx_mlp_backward / training step, same layout as the parameters. */
int nfx_mlp_get_grads(nfx_mlp* mlp, float* grads);
/* y[batch x n_out] = f(x[batch x n_in]). */
int nfx_mlp_forward(nfx_mlp* mlp, const float* x, int64_t batch, float* y);
/* Loss L = scale * sum_b w_b * ||f(x_b) - target_b||^2 (w = 1 when weight is NULL): per-row
 * losses w_b * ||.||^2 into loss[batch] (nullable), the parameter gradients of L kept for
 * nfx_mlp_adamw / nfx_mlp_get_grads, and dL/dx into dx[batch x n_in] when dx is not NULL. */
int nfx_mlp_backward(nfx_mlp* mlp, const float* x, const float* target, const float* weight, int64_t batch,
                     float scale, float* loss, float* dx);
/* One AdamW update of every parameter from the stored gradients (decoupled weight decay on the
 * weights, not on the biases). */
int nfx_mlp_adamw(nfx_mlp* mlp, float lr, float beta1, float beta2, float eps, float weight_decay);
/* steps minibatch steps over a dataset of n rows uploaded once (x[n x n_in], target[n x n_out],
 * weight[n] nullable): PCG32-shuffled epochs (seed), mean weighted squared-error loss, AdamW with
 * a cosine learning rate from hp[0] to hp[5]; hp = {lr, beta1, beta2, eps, weight_decay, lr_min}.
 * losses[steps] (nullable) receives each step's mean loss. */
int nfx_mlp_train(nfx_mlp* mlp, const float* x, const float* target, const float* weight, int64_t n, int64_t batch,
                  int64_t steps, const float* hp, uint64_t seed, float* losses);
/* Inverse problem: Adam on the inputs of `batch` rows to minimise w_b * ||f(x_b) - target_b||^2;
 * only inputs with free_mask[k] != 0 move, all stay in [lo[k], hi[k]]. x is updated in place;
 * loss[batch] (nullable) gets the final per-row loss. hp = {lr, beta1, beta2, eps}. */
int nfx_mlp_fit_inputs(nfx_mlp* mlp, float* x, const float* target, const float* weight, int64_t batch,
                       const unsigned char* free_mask, const float* lo, const float* hi, int64_t steps,
                       const float* hp, float* loss);

#ifdef __cplusplus
}
#endif

#endif /* NFX_H */
