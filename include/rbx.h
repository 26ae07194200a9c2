/*
 * rbx.h -- C ABI of the GB300-native rigid-body integrator (librbx.so).
 *
 * The library replaces the compute path of the OpenMM rigid-body plugin's
 * CudaIntegrateRigidBodyStepKernel (platforms/cuda/src/CudaRigidBodyKernels.cpp) and the
 * host-side RigidBodySystem (openmmapi/src/RigidBodySystem.cpp) it feeds. Every entry point
 * takes plain pointers and sizes; device pointers are borrowed from the caller (an OpenMM
 * CudaContext, or any CUDA allocation with the same layout) and never freed by the library.
 * All calls return RBX_OK (0) or a non-zero rbx_status; rbx_last_error() gives the message of
 * the calling thread's last failure.
 *
 * Device buffer layout (OpenMM CUDA platform conventions):
 *   posq            float4 (single, mixed) or double4 (double) per atom slot; .w (charge) kept
 *   posq_correction float4 per slot, mixed precision only (position = posq + correction)
 *   velm            float4 (single) or double4 (mixed, double); .w = 1/mass, kept
 *   force           long long, fixed point with scale 2^32, SoA: x at [slot], y at
 *                   [slot + stride], z at [slot + 2*stride]; read only
 * Atom i of the user's System lives in device slot location[i] (identity unless
 * rbx_set_atom_locations says otherwise, mirroring OpenMM's atom reordering).
 */
#ifndef RBX_H
#define RBX_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rbx_integrator rbx_integrator;

enum rbx_precision { RBX_PRECISION_SINGLE = 0, RBX_PRECISION_MIXED = 1, RBX_PRECISION_DOUBLE = 2 };

enum rbx_status {
    RBX_OK = 0,
    RBX_ERR_INVALID_ARGUMENT = 1, /* OpenMMException for misuse in the reference */
    RBX_ERR_CUDA = 2,             /* a CUDA runtime call failed */
    RBX_ERR_STATE = 3,            /* call order violated (e.g. step before rbx_upload_state) */
    RBX_ERR_UNSUPPORTED = 4,      /* feature outside this build (e.g. body larger than a tile) */
    RBX_ERR_NUMERIC = 5           /* non-finite result detected */
};

/* Device buffers of one OpenMM-style context (borrowed). */
typedef struct rbx_buffers {
    void* posq;
    void* posq_correction; /* NULL unless mixed precision */
    void* velm;
    const long long* force;
    int stride; /* force SoA stride (OpenMM paddedNumAtoms), >= number of atom slots */
} rbx_buffers;

/* Message of this thread's last failure ("" if none). */
const char* rbx_last_error(void);
/* ABI version of this build (major*10000 + minor*100 + patch). */
int rbx_version(void);

/*
 * Create the integrator kernel for a System of num_atoms atoms.
 * Replaces RigidBodyIntegrator(stepSize, bodyIndices) + setRotationMode
 * (openmmapi/src/RigidBodyIntegrator.cpp:18-32), RigidBodySystem::initialize
 * (openmmapi/src/RigidBodySystem.cpp:55-114) and CudaIntegrateRigidBodyStepKernel::initialize
 * (platforms/cuda/src/CudaRigidBodyKernels.cpp:232-288).
 *   body_indices  [num_atoms]: 0 (or negative) = free atom; atoms sharing a positive index form
 *                 one rigid body. An index used by a single atom makes that atom free.
 *   masses        [num_atoms] in amu; massless atoms may only be free (they are not moved).
 *   rotation_mode 0 = exact (Jacobi elliptic), n > 0 = NO-SQUISH with n substeps.
 *   precision     enum rbx_precision; device = CUDA device ordinal.
 * Errors: RBX_ERR_INVALID_ARGUMENT for a negative mode (RigidBodyIntegrator.cpp:28-29), a bad
 * count, or a massless body atom. RBX_ERR_UNSUPPORTED for a body larger than a tile (1024 atoms
 * in single and mixed precision, 512 in double) or a system beyond 32-bit device indexing (about
 * 76 million bodies, or 715 million body atoms or free atoms; the buffer stride likewise).
 */
int rbx_create(rbx_integrator** out, int num_atoms, const int* body_indices, const double* masses,
               int rotation_mode, int precision, int device);
int rbx_destroy(rbx_integrator* h);

/* Map user atom i -> device slot location[i] (OpenMM atom reordering; replaces the
 * ReorderListener's atomLocation rebuild, CudaRigidBodyKernels.cpp:69-113). Slots must be
 * non-negative and distinct (RBX_ERR_INVALID_ARGUMENT otherwise, and nothing changes). The library
 * keeps its device arrays with bodies ordered by the lowest slot of their atoms and free atoms by
 * slot (so that a CTA's atoms occupy a narrow slot range); this call re-plans that order on the
 * device (a counting sort over slots) and moves every per-body and per-atom array to it bit for
 * bit (8.4 ms for 1e6 bodies and 1e5 free atoms on GB300). Synchronous. */
int rbx_set_atom_locations(rbx_integrator* h, const int* location);

/*
 * Build the rigid-body state from atom positions and velocities (host arrays, user order,
 * [num_atoms*3] doubles) and upload it. Replaces RigidBodySystem::update
 * (RigidBodySystem.cpp:120-142) with RigidBody::buildGeometry/buildDynamics
 * (openmmapi/src/RigidBody.cpp:65-142) and uploadBodySystem (CudaRigidBodyKernels.cpp:293-372).
 * Uses a robust eigensolver; body velocities are projected onto rigid motion.
 */
int rbx_upload_state(rbx_integrator* h, const double* positions, const double* velocities);

/*
 * Body setup on the device, from the positions, velocities (and the masses given to rbx_create) of
 * the atoms already in `buf` at their device slots: the same robust setup as rbx_upload_state, the
 * same arithmetic (bit-identical results), without copying positions and velocities to the host.
 * Replaces RigidBodySystem::update + uploadBodySystem on a state change
 * (RigidBodyIntegrator.cpp:63-74, CudaRigidBodyKernels.cpp:293-372). Synchronises `stream`.
 */
int rbx_upload_state_device(rbx_integrator* h, void* stream, const rbx_buffers* buf);

/* Counts: RigidBodySystem::getNumDOF/getNumBodies/getNumFree (RigidBodySystem.h:38-42). */
int rbx_get_num_dof(const rbx_integrator* h, int* out);
int rbx_get_num_bodies(const rbx_integrator* h, int* out);
int rbx_get_num_free(const rbx_integrator* h, int* out);
int rbx_get_rotation_mode(const rbx_integrator* h, int* out);
/*
 * The degrees of freedom exactly as the reference counts them, numFree - numConstraints + sum of
 * body dof (openmmapi/src/RigidBodySystem.cpp:130), for callers that must report the plugin's own
 * integer (its getNumDOF, and the temperature of its StateDataReporter, python/statedatareporter.py:
 * 19-28). It differs from rbx_get_num_dof in two ways:
 *   - a free atom counts 1, not 3;
 *   - an atom whose body index is used once is a one-atom body in the reference (cleanBodyIndices
 *     keeps it, RigidBodySystem.cpp:37-47) and counts 5 or 6: 6 when its displacement from its own
 *     centre of mass, x - (x m)(1/m), is zero in every component, 5 when rounding leaves a residue
 *     that the collinearity test then accepts (RigidBody.cpp:26-45, :88-107). It is evaluated on the
 *     positions of the last rbx_upload_state / rbx_upload_state_device, as the reference evaluates it
 *     on every state update. Massless atoms count nothing.
 * RBX_ERR_STATE before the first state upload.
 */
int rbx_get_num_dof_reference(const rbx_integrator* h, int* out);

/*
 * Tile shape of the single/mixed step kernel (no counterpart in the reference, which launches
 * fixed 128-thread blocks, CudaRigidBodyKernels.cpp:135-139): 256 threads per tile of at most 256
 * bodies and 1024 body atoms (the default, 3 tiles resident per SM) or 128 threads per tile of at
 * most 128 bodies and 512 body atoms (6 per SM). Results are identical, bit for bit, under either;
 * only the speed differs. RBX_ERR_UNSUPPORTED for 128 threads when a body has more than 32 atoms
 * (such bodies are summed by a whole warp, in a form of the kernel built for 256 threads only), or
 * in double precision (one shape: 256 threads, 512 body atoms). Waits for the device; call it
 * between steps, not during a stream capture.
 */
int rbx_set_tile_threads(rbx_integrator* h, int threads);
int rbx_get_tile_threads(const rbx_integrator* h, int* out);

/*
 * One half of a step on OpenMM-layout device buffers, enqueued on `stream` (cudaStream_t,
 * NULL = default stream). Replaces the integrateRigidBodyPart1 / integrateRigidBodyPart2
 * kernels and freeAtomsDelta (platforms/cuda/src/kernels/rigidbodyintegrator.cu:270-396)
 * launched by CudaIntegrateRigidBodyStepKernel::execute (CudaRigidBodyKernels.cpp:377-444).
 *   part1: half kick by the forces in `force`, drift, free rotation, atom positions.
 *   part2: half kick by the forces in `force`, atom velocities.
 *   fused: part2 of step n followed by part1 of step n+1 in one pass; atom velocities of body
 *          atoms are not written (call part2 to synchronise them).
 * A full step is part1, force evaluation, part2.
 */
int rbx_integrate_part1(rbx_integrator* h, void* stream, const rbx_buffers* buf, double dt);
int rbx_integrate_part2(rbx_integrator* h, void* stream, const rbx_buffers* buf, double dt);
int rbx_integrate_fused(rbx_integrator* h, void* stream, const rbx_buffers* buf, double dt);

/*
 * Constraints between free atoms (bond-length constraints that OpenMM's solvers enforce).
 * rbx_set_constraints checks the System's constraints, atom pairs [2*num_constraints], as
 * RigidBodySystem::initialize does (openmmapi/src/RigidBodySystem.cpp:107-113: "Constraints
 * involving rigid-body atoms are not allowed"); each removes one degree of freedom
 * (RigidBodySystem.cpp:130).
 * A step with constrained free atoms replaces rbx_integrate_part1 by three calls, the protocol of
 * CudaRigidBodyKernels.cpp:405-419 around OpenMM's posDelta buffer (mixed4 per slot: float4 in
 * single precision, double4 in mixed and double):
 *   rbx_free_atoms_delta      pos_delta <- h (v + F/m h/2) for every free atom (freeAtomsDelta,
 *                             rigidbodyintegrator.cu:270-279);
 *   (OpenMM's applyConstraints corrects pos_delta);
 *   rbx_integrate_part1_delta bodies as rbx_integrate_part1; free atoms move by the corrected
 *                             pos_delta and take it over h as their mid-step velocity.
 * Then forces, rbx_integrate_part2 and OpenMM's applyVelocityConstraints. The velocity follows the
 * Reference platform (RigidBodySystem.cpp:172-176, :197: the (R - savedPos)/dt correction after
 * SHAKE); the CUDA reference saves the position after the constraints, so its correction is zero.
 * Fused steps skip the constraints and must not be used with them. Refined energies are not
 * available with constrained free atoms (RBX_ERR_UNSUPPORTED).
 */
int rbx_set_constraints(rbx_integrator* h, int num_constraints, const int* atom_pairs);
int rbx_free_atoms_delta(rbx_integrator* h, void* stream, const rbx_buffers* buf, void* pos_delta, double dt);
int rbx_integrate_part1_delta(rbx_integrator* h, void* stream, const rbx_buffers* buf, const void* pos_delta,
                              double dt);

/*
 * Failure detector. The reference produces NaN silently when its exact rotation fails
 * (openmmapi/include/internal/ellipticFunctions.h:38-39, :64-66) and keeps stepping it. Here every
 * step kernel checks the new state of each body and free atom for a non-finite value (one sum of
 * values it holds anyway) and flags the ones that fail. rbx_check_state synchronises `stream` and
 * returns RBX_ERR_NUMERIC, with the counts of flagged bodies and free atoms (either pointer may be
 * NULL) and a message naming the first of each (bodies in ascending body-index order, free atoms by
 * user index), when any step since the last state change failed; RBX_OK and zero counts otherwise.
 * The flags are cleared by rbx_upload_state, rbx_upload_state_device and rbx_set_body_state.
 */
int rbx_check_state(rbx_integrator* h, void* stream, int* bad_bodies, int* bad_free);

/*
 * Translational and rotational kinetic energy [KE_t, KE_r] in kJ/mol, reduced on the device in
 * FP64 in a fixed order; synchronises `stream`. Replaces the kineticEnergies kernel plus host
 * summation (rigidbodyintegrator.cu:416-427, CudaRigidBodyKernels.cpp:118-163) and
 * RigidBodySystem::computeKineticEnergies (RigidBodySystem.cpp:210-220).
 */
int rbx_kinetic_energies(rbx_integrator* h, void* stream, const rbx_buffers* buf, double* out2);

/*
 * Refined ("shadow") energies. Replaces RigidBodyIntegrator::setComputeRefinedEnergies
 * (openmmapi/src/RigidBodyIntegrator.cpp:34-38), which compiles the plugin's kernels with
 * COMPMOD = 1 (CudaRigidBodyKernels.cpp:240); getRefinedKineticEnergies
 * (CudaRigidBodyKernels.cpp:469-476, :118-163; refinedKineticEnergies kernel,
 * rigidbodyintegrator.cu:433-443) and getPotentialEnergyRefinement (CudaRigidBodyKernels.cpp:
 * 481-494, :168-194; potentialEnergyRefinement kernel, rigidbodyintegrator.cu:449-469).
 *
 * While on, every part1 / fused step starts and every part2 closes the stencils of the reference
 * (rigidbodyintegrator.cu:238-243, :285-292, :318-321, :380-384): after part2 of step n,
 *   refined KE_t = sum over bodies and free atoms of m v . s / (6h) (s/2 for free atoms),
 *   refined KE_r = sum over bodies of qdot . pi / (6h),
 *   U_refinement = -h^2/24 (sum |F|^2/m + tau . I^-1 . tau),
 * with s and qdot the position and quaternion stencils over t-h .. t+2h. Free atoms use the
 * stencil weights of the bodies (-1, 5, 2 on the three half-step displacements); the reference's
 * free-atom path weights the first +1, which reports 4/3 of the kinetic energy for uniform motion.
 * Sums are FP64 in a fixed order; the kernels write per-body corrections to the plain kinetic
 * energy, so nothing is lost to cancellation in the FP32 paths.
 * Off (the default): rbx_refined_kinetic_energies returns the plain kinetic energies and
 * rbx_potential_energy_refinement 0, as the reference does. On, both need a completed step (part1
 * or fused, then part2, same step size) since the last state change (RBX_ERR_STATE otherwise).
 * Switching it on allocates 28-56 bytes per body and 12-24 per free atom; the step kernels then
 * read and write them (the plain step is unchanged while it is off). Both queries synchronise
 * `stream`.
 */
int rbx_set_compute_refined_energies(rbx_integrator* h, int compute);
int rbx_get_compute_refined_energies(const rbx_integrator* h, int* out);
int rbx_refined_kinetic_energies(rbx_integrator* h, void* stream, const rbx_buffers* buf, double* out2);
int rbx_potential_energy_refinement(rbx_integrator* h, void* stream, const rbx_buffers* buf, double* out1);

/*
 * Body state exchange for tests and checkpoints, host arrays with bodies in the reference's
 * order (ascending body index, as RigidBodySystem numbers them; RigidBodySystem.cpp:28-49):
 *   state [num_bodies*14]: r[3], v[3], q[4], pi[4] per body (v = centre-of-mass velocity)
 *   geometry [num_bodies*3] principal moments I (descending; I[2] = 0 for a linear body)
 * rbx_get_body_atoms gives the first body atom of each body [nb+1] and, for body-atom k, the
 * user atom index [nba], in the same order; body_fixed follows that atom order.
 */
int rbx_get_body_state(rbx_integrator* h, double* state);
int rbx_set_body_state(rbx_integrator* h, const double* state);
/* The body state's exact device words, for checkpoints: 112 bytes per body in every precision, in
 * the same body order: 14 doubles (double precision), or the 14 high then the 14 low floats of the
 * float-float state (single, mixed). A float-float pair summed into one double loses the low word's
 * last bits when it is below 2^-29 of the high word, so the double rows of rbx_get_body_state do
 * not restore such a state bit for bit; these rows do. */
int rbx_get_body_state_raw(rbx_integrator* h, void* rows);
int rbx_set_body_state_raw(rbx_integrator* h, const void* rows);
int rbx_get_body_geometry(rbx_integrator* h, double* moments, double* body_fixed /* [nba*3] */);
int rbx_get_body_atoms(rbx_integrator* h, int* first_atom /* [nb+1] */, int* atoms /* [nba] */);

/*
 * Host-buffer step, the counterpart of the Reference platform's step on host vectors
 * (RigidBodySystem::integratePart1/integratePart2, RigidBodySystem.cpp:170-204):
 * copies `forces` ([num_atoms*3] doubles, user order, pinned memory recommended) to the device,
 * runs `nsteps` steps with that fixed force array (part1, fused x (nsteps-1), part2) on buffers
 * owned by the integrator, and copies the resulting positions and velocities back into
 * `positions`/`velocities` ([num_atoms*3]). Synchronous on `stream`.
 * rbx_context_set_state loads the owned buffers from host positions/velocities and builds the
 * body state (rbx_upload_state); rbx_context_buffers exposes the owned device buffers.
 */
int rbx_context_set_state(rbx_integrator* h, void* stream, const double* positions, const double* velocities);
int rbx_context_buffers(rbx_integrator* h, rbx_buffers* out);
int rbx_context_set_forces(rbx_integrator* h, void* stream, const double* forces);
int rbx_context_get_state(rbx_integrator* h, void* stream, double* positions, double* velocities);
/* Exact restore of a saved state (no counterpart in the reference, which rebuilds its bodies from
 * the Context's positions on every state change, RigidBodyIntegrator.cpp:63-74):
 * rbx_context_load writes host positions and velocities into the owned buffers as they are, without
 * rebuilding the body state; rbx_context_sync_bodies rewrites the body atoms' positions from the
 * current body state with the step kernels' own arithmetic. With rbx_set_body_state_raw in
 * between, a state saved by rbx_get_body_state_raw + rbx_context_get_state is restored bit for bit. */
int rbx_context_load(rbx_integrator* h, void* stream, const double* positions, const double* velocities);
/* rbx_context_get_state for the user atoms [first_atom, first_atom + count) only. */
int rbx_context_get_range(rbx_integrator* h, void* stream, int first_atom, int count, double* positions,
                          double* velocities);
int rbx_context_sync_bodies(rbx_integrator* h, void* stream);
int rbx_step_host(rbx_integrator* h, void* stream, int nsteps, double dt, const double* forces, double* positions,
                  double* velocities);

/*
 * Allocation-free kinetic energy. This entry point has no counterpart in the reference plugin.
 *
 * For callers that cannot call cudaMalloc: a serving process that has reserved its whole
 * device-memory budget up front and admits work only against that reservation, a host framework
 * whose own pool owns every device allocation, or a latency-sensitive loop that cannot take the
 * device synchronisation an allocation may cause. It computes [KE_t, KE_r] from caller-owned
 * device arrays; the results agree with rbx_kinetic_energies to rounding (about 1e-12 relative:
 * the two reductions partition their sums differently) and are identical from call to call on
 * the same inputs. It allocates nothing: no cudaMalloc,
 * no cudaFree, no allocating library call. Its scratch (block partial sums and a ticket counter)
 * is a fixed static device array of 16 KB + 256 B that every GPU which loads librbx holds until
 * the process exits.
 *   body_state   [14 * body_stride] FP64 rows r.xyz, v.xyz, q.wxyz, pi.wxyz (the state layout of
 *                rbx_get_body_state, transposed to rows of body_stride)
 *   inv_mass     [num_bodies] 1/m; inv_inertia [3 * body_stride] rows of 1/I (0 for the axis of a
 *                linear body)
 *   velm         device velm array (float4 for single, double4 otherwise); free_slots
 *                [num_free] device slot of each free atom (a slot whose velm.w = 1/m is 0, a
 *                massless particle, contributes nothing)
 *   out_device   device double[2] receiving [KE_t, KE_r] (kJ/mol); asynchronous on `stream`.
 * Limit: at most 4,194,304 bodies and 4,194,304 free atoms (1024 block sums of 4096 items), and
 * body_stride * 14 within 32-bit indexing; larger inputs get RBX_ERR_UNSUPPORTED. Each call
 * outside stream capture looks up the scratch address on the current device (so a device reset,
 * which reloads the module, is followed); a call on a capturing stream reuses the address of the
 * last call on that device, so make the first call on a device before any stream capture. All calls
 * share the one scratch array, so calls that overlap on the GPU (concurrent streams, several host
 * threads) race and must be serialised by the caller.
 */
int rbx_kinetic_energies_static(const double* body_state, int num_bodies, int body_stride, const double* inv_mass,
                                const double* inv_inertia, const void* velm, const int* free_slots, int num_free,
                                int precision, void* stream, double* out_device);

/*
 * Pipelined rbx_step_host: the same work (forces in, nsteps steps, positions and velocities out),
 * asynchronous. Consecutive calls overlap one call's force upload and another's result download
 * with a third's kernels (double-buffered device staging, internal copy streams ordered by
 * events); the kernels run on `stream`. The host arrays must stay untouched until the results
 * are waited for, and should be pinned (pageable memory makes the copies synchronous).
 * rbx_step_host_wait blocks until every result of earlier calls is in its host arrays.
 */
int rbx_step_host_async(rbx_integrator* h, void* stream, int nsteps, double dt, const double* forces,
                        double* positions, double* velocities);
int rbx_step_host_wait(rbx_integrator* h);

/* Number of kernel launches the last integrate/kinetic/step call enqueued (for accounting). */
int rbx_last_launch_count(const rbx_integrator* h);

/*
 * Batched systems: many independent periodic systems integrated together, with forces from the
 * library's own cutoff Lennard-Jones + reaction-field kernel (the functional form of OpenMM's
 * NonbondedForce with the CutoffPeriodic method; pairs of one rigid body excluded, as the
 * plugin's ForceField helper removes them, python/forcefield.py:131-138). The reference has no
 * batched form: each system of the reference is one Context with one integrator kernel, stepped
 * by RigidBodyIntegrator::step (RigidBodyIntegrator.cpp:76-93) -> execute
 * (CudaRigidBodyKernels.cpp:377-444); this handle runs that same step for every system at once.
 *
 *   num_systems   S; system s holds atoms [atom_offsets[s], atom_offsets[s+1]) of the arrays
 *   box_edges     [S] cubic box edge (nm); cutoffs [S] cutoff (nm), each below box_edges[s]/2
 *   body_indices  [N] per-system body ids (0 = free atom; equal positive ids within a system
 *                 form one rigid body, as in rbx_create)
 *   masses, charges (e), sigmas (nm), epsilons (kJ/mol)  [N]; Lorentz-Berthelot combination
 *   eps_solvent   reaction-field dielectric (OpenMM's default is 78.3)
 * Atoms live in device slots equal to their index in these arrays.
 * rbx_batch_step runs nsteps velocity-Verlet steps of size dt on every system: forces at the
 * current positions, part1, then (forces, fused part2+part1) x (nsteps-1), forces, part2. The
 * forces at the starting positions are those the previous rbx_batch_step ended with when no other
 * call has changed the state since (one force evaluation per step, as the reference's execute
 * keeps the last step's forces, CudaRigidBodyKernels.cpp:421-426); otherwise the call forms them
 * first. With
 * rbx_batch_set_graph_steps(k > 0), runs of k (forces, fused) pairs replay one captured CUDA graph
 * (captured on first use for a given dt; invalidated by rbx_batch_set_state).
 * rbx_batch_energies returns [U, KE_t, KE_r] per system (kJ/mol) at the current state
 * (synchronous); U comes from the last force evaluation of the preceding rbx_batch_step when no
 * other call has changed the state since. rbx_batch_get_num_dof gives each system's degrees of
 * freedom.
 * Forces come from neighbour lists of atom groups (each rigid body is one group, each free atom a
 * group of its own): two groups are listed together when their centroids lie within cutoff + a
 * skin of 0.06 nm + both groups' radii. Each system rebuilds its lists when one of its centroids has
 * moved half the skin, and every list is rebuilt for the state a step call ends in (and for the
 * first evaluation after rbx_batch_set_state or rbx_batch_restore), so the forces and energy at a
 * call's start and end depend on the positions alone: a system's results are a function of its own
 * state and of the lengths of the calls that step it.
 */
typedef struct rbx_batch rbx_batch;
/* rbx_batch_set_state builds every body from the given positions and velocities (as
 * rbx_upload_state does) and then places the body atoms where the body state puts them. */
int rbx_batch_create(rbx_batch** out, int num_systems, const int* atom_offsets, const double* box_edges,
                     const double* cutoffs, const int* body_indices, const double* masses, const double* charges,
                     const double* sigmas, const double* epsilons, double eps_solvent, int rotation_mode,
                     int precision, int device);
int rbx_batch_destroy(rbx_batch* b);
int rbx_batch_set_state(rbx_batch* b, void* stream, const double* positions, const double* velocities);
int rbx_batch_get_state(rbx_batch* b, void* stream, double* positions, double* velocities);
/* Positions and velocities of system s only ([n_s*3] each). */
int rbx_batch_get_system_state(rbx_batch* b, void* stream, int s, double* positions, double* velocities);
/* Checkpoint and exact restore. rbx_batch_get_body_state gives every body's state as the exact
 * rows of rbx_get_body_state_raw (112 bytes per body; bodies system by system in ascending body
 * index). After rbx_batch_set_state with the positions the saved batch was last set up from (they
 * fix each body's principal frame and body-frame coordinates), rbx_batch_restore puts back saved
 * body rows, positions and velocities bit for bit. */
int rbx_batch_get_body_state(rbx_batch* b, void* body_rows);
int rbx_batch_restore(rbx_batch* b, void* stream, const void* body_rows, const double* positions,
                      const double* velocities);
int rbx_batch_step(rbx_batch* b, void* stream, int nsteps, double dt);
/* Relaxation by damped dynamics: nsteps times (forces capped at max_force kJ/mol/nm per atom,
 * every momentum scaled by `damping` in [0, 1), part1 of size dt), then every momentum zeroed.
 * Removes the overlaps of generated starting structures before dynamics; velocities are then
 * reassigned by rbx_batch_set_state. Not a step of the reference, which takes its starting state
 * as given. */
int rbx_batch_relax(rbx_batch* b, void* stream, int nsteps, double dt, double max_force, double damping);
int rbx_batch_energies(rbx_batch* b, void* stream, double* out /* [3*S] */);
int rbx_batch_forces(rbx_batch* b, void* stream, double* forces /* [N*3], user order */, double* energies /* [S] */);
int rbx_batch_get_num_dof(rbx_batch* b, int* dof /* [S] */);
/* Failure status per system (no counterpart in the reference, which has no batched form and lets
 * NaN through silently). A system fails when a step leaves any of its bodies or free atoms with a
 * non-finite state (the step kernels' detector, see rbx_check_state) or when the force kernel
 * meets a non-finite force or one beyond OpenMM's fixed-point range (|F| >= 2^31 kJ/mol/nm, i.e.
 * overlapping atoms). Synchronises `stream`; system_status [S] (may be NULL) receives RBX_OK or
 * RBX_ERR_NUMERIC per system, num_failed (may be NULL) their number. Returns RBX_ERR_NUMERIC,
 * naming the first failed system, when any failed. Systems are independent: a failed system
 * changes nothing for the others, which keep stepping exactly as they would alone. The status is
 * cleared by rbx_batch_set_state and rbx_batch_restore. */
int rbx_batch_status(rbx_batch* b, void* stream, int* system_status, int* num_failed);
/* Device memory the batch holds: every allocation of the batch and of its integrator, in bytes as
 * requested from cudaMalloc (no counterpart in the reference). A serving loop admits work against
 * this figure and the device's free memory. Grows when a later call allocates lazily (the first
 * rbx_batch_set_state, CUDA-graph capture aside, which the driver allocates). */
int rbx_batch_memory(const rbx_batch* b, size_t* bytes);
/* Neighbour-list builds of each system since the batch was created (counts [S]; synchronises
 * `stream`): a statistic of the force path (no counterpart in the reference). */
int rbx_batch_list_builds(rbx_batch* b, void* stream, unsigned int* counts);
int rbx_batch_set_graph_steps(rbx_batch* b, int k);
/* Autotuner of the batched step's schedule (no counterpart in the reference, which has no batched
 * form). It times, on the batch itself and with direct launches:
 *   1. the step kernel's tile shape (rbx_set_tile_threads: 256 or 128 threads, single/mixed
 *      precision with bodies of at most 32 atoms), by the integrator launches' own event times
 *      over 2 x trial_steps steps after an untimed run of trial_steps;
 *   2. the block size of the cell list-build kernel (64, 128 or 256 threads per cell);
 *   3. where a step takes under 1 ms, so that launch overhead matters, the steps per captured graph
 *      (0, 10 or 50).
 * Trials 2 and 3 run trial_steps steps (2k+1 for a graph of k) twice and time the second run with
 * CUDA events. It keeps the fastest of each, and then restores the batch's exact state
 * (rbx_batch_restore): no choice changes any result, since each body is integrated alike in any
 * tile, each group's list (and so each atom's force sum) keeps its order, and graphs replay the
 * same launches.
 * chosen[2] (optional) receives the block size and the graph run length; rbx_batch_get_tile_threads
 * the tile shape. rbx_batch_set_tuning and rbx_batch_set_tile_threads set them by hand. */
int rbx_batch_autotune(rbx_batch* b, void* stream, double dt, int trial_steps, int* chosen);
int rbx_batch_set_tuning(rbx_batch* b, int cell_threads, int graph_steps);
int rbx_batch_set_tile_threads(rbx_batch* b, int threads);
int rbx_batch_get_tile_threads(rbx_batch* b, int* out);
/* Event timing of the force and integrator launch groups of later calls (direct launches only:
 * graphs are not used while timing is on); rbx_batch_kernel_times waits for and sums them
 * (milliseconds) and starts a new tally. */
int rbx_batch_set_timing(rbx_batch* b, int on);
int rbx_batch_kernel_times(rbx_batch* b, double* ms_forces, double* ms_integrator, int* groups);
int rbx_batch_last_launch_count(const rbx_batch* b);

#ifdef __cplusplus
}
#endif
#endif /* RBX_H */
