/* C ABI of the GB300 MPIDForce evaluation (libmpid_gb300.so).
 *
 * This is the drop-in boundary for the reference's platform kernel
 * CalcMPIDForceKernel (openmmapi/include/openmm/mpidKernels.h:50-104): a context holds
 * one MPIDForce's parameters on one GPU and evaluates energy, forces and induced
 * dipoles under PME (or no cutoff) with Direct, Mutual or Extrapolated polarisation.
 * Plain pointers and sizes only; no exceptions cross the boundary.  Every function
 * returns MPID_OK (0) or a negative status; mpid_last_error() gives the message of the
 * last failure on the calling thread.
 *
 * Units: nm, e, kJ/mol.  Atom order is the caller's; the library sorts internally.
 * Parameter orders follow MPIDForce::addMultipole (openmmapi/include/openmm/MPIDForce.h:245):
 *   dipole X Y Z; quadrupole XX XY YY XZ YZ ZZ;
 *   octopole XXX XXY XYY YYY XXZ XYZ YYZ XZZ YZZ ZZZ.
 */
#ifndef MPID_GB300_H
#define MPID_GB300_H
#ifdef __cplusplus
extern "C" {
#endif

#define MPID_OK 0
#define MPID_ERR_INVALID -1        /* invalid argument or parameter (MPIDForceImpl.cpp:56-150) */
#define MPID_ERR_CUDA -2           /* CUDA / cuFFT failure */
#define MPID_ERR_NOT_CONVERGED -3  /* mutual induced dipoles did not converge (MPIDReferenceForce.cpp:2229-2235) */
#define MPID_ERR_STATE -4          /* call made before the required set-up */

/* Nonbonded methods and polarisation types: values of MPIDForce::NonbondedMethod and
 * MPIDForce::PolarizationType (MPIDForce.h:58-94). */
#define MPID_NO_CUTOFF 0
#define MPID_PME 1
#define MPID_MUTUAL 0
#define MPID_DIRECT 1
#define MPID_EXTRAPOLATED 2

/* Arithmetic of the evaluation. */
#define MPID_PRECISION_MIXED 0   /* FP32 pair/PME/solver, 64-bit fixed-point forces, FP64 energy and refinement */
#define MPID_PRECISION_DOUBLE 1  /* FP64 throughout */

/* mpid_settings.flags */
#define MPID_FLAG_EXACT_ANISO_TORQUE 1u  /* use the energy-consistent induced-induced torque on
                                            anisotropic atoms instead of the reference's */
#define MPID_FLAG_NEAR_FIELD_PCG 2u      /* mutual solver preconditioned with the near-field dipole
                                            coupling (fewer iterations for strongly coupled systems;
                                            on water it saves one iteration and costs more) */
#define MPID_FLAG_GRAPH_SOLVER 4u        /* PME: evaluation segments and mutual-solver iterations
                                            replayed from CUDA graphs captured once per neighbour-list
                                            shape and box (small systems, where launches cost more than
                                            the work); on the legacy default stream they run directly */
#define MPID_FLAG_SERIAL_STAGES 8u       /* profiling: the context's side streams (PME chains, the FP64
                                            residual check) fold onto the caller's stream, so that the
                                            stage times of mpid_stats add up to the evaluation's device
                                            time, and cuFFT executions are timed as their own stage (4);
                                            slower than the default overlapped schedule, same results */

typedef struct mpid_context mpid_context;

/* Force-wide settings; the fields mirror MPIDForce's getters/setters
 * (MPIDForce.h:106-232, defaults MPIDForce.cpp:43-50). */
typedef struct {
    int num_atoms;
    int nonbonded_method;      /* MPID_PME or MPID_NO_CUTOFF */
    int polarization_type;     /* MPID_MUTUAL, MPID_DIRECT, MPID_EXTRAPOLATED */
    double cutoff;             /* nm (PME) */
    double ewald_alpha;        /* nm^-1, must be > 0 for PME */
    int grid[3];               /* PME grid, each > 0 for PME */
    int pme_order;             /* 5 or 6 (the reference fixes 6) */
    double mutual_eps;         /* Debye RMS target of the mutual solver */
    int max_iter;              /* mutual solver iteration limit */
    int n_extrap;              /* number of extrapolation coefficients (<= 8) */
    double extrap_coeffs[8];
    double default_thole;      /* MPIDForce::setDefaultTholeWidth */
    double scale14;            /* MPIDForce::set14ScaleFactor */
    int precision;             /* MPID_PRECISION_MIXED or MPID_PRECISION_DOUBLE */
    unsigned flags;
} mpid_settings;

/* Per-evaluation statistics. */
typedef struct {
    int solver_iterations;     /* FP32/FP64 CG iterations (mutual), PT orders (extrapolated) */
    int refinement_steps;      /* FP64 residual evaluations (mixed mutual) */
    double solver_residual;    /* final Debye RMS residual */
    int max_neighbours;        /* longest per-atom neighbour list of the last evaluation */
    double ms_total;           /* device time of the last evaluation */
    /* device time (ms) and timed launch groups per stage: 0 sort/tiles/atom set-up,
     * 1 permanent-field pair kernel, 2 PME spread/FFT/convolution/gather (without the FFTs
     * under MPID_FLAG_SERIAL_STAGES), 3 dipole-field pair kernels, 4 cuFFT executions (timed
     * only under MPID_FLAG_SERIAL_STAGES; otherwise inside stage 2), 5 energy/force/torque
     * pair kernel, 6 reciprocal/self terms and torque mapping, 7 FP64 dipole-field pair
     * kernel of the mixed path's residual refinement.  The solver's vector kernels are not
     * timed as a stage.  Stages on different streams overlap unless MPID_FLAG_SERIAL_STAGES
     * is set, and inside replayed graphs a stage's time includes its waits for other
     * streams, so only the serial stage times add up to ms_total. */
    double ms_stage[8];
    int stage_launches[8];
    double energy_parts[3];    /* reciprocal + self, real-space pairs, covalently scaled pairs */
    int kernel_launches;       /* launches of this library's kernels in the last evaluation
                                  (with its gradient passes, mpid_evaluate_with_gradients) */
    int library_calls;         /* cuFFT executions and cub sorts, counted the same way */
    int graph_captures;        /* CUDA graphs captured by the last evaluation and its gradients */
    int graph_replays;         /* graph launches of the last evaluation and its gradients */
    long long device_allocations; /* cudaMalloc calls made by this library in this process so far
                                     (all contexts; read when mpid_get_stats is called) */
} mpid_stats;

/* Fill `s` with the MPIDForce defaults for n atoms (PME not configured). */
void mpid_default_settings(mpid_settings* s, int num_atoms);

/* Create a context on CUDA device `device`.  Replaces
 * CudaCalcMPIDForceKernel::initialize (platforms/cuda/src/MPIDCudaKernels.cpp:210-662)
 * and the validation of MPIDForceImpl::initialize (openmmapi/src/MPIDForceImpl.cpp:51-150). */
int mpid_create(const mpid_settings* settings, int device, mpid_context** out);
void mpid_destroy(mpid_context* ctx);

/* Multipole parameters of every atom (MPIDForce::addMultipole / setMultipoleParameters,
 * MPIDForce.h:245-282); validated as MPIDForceImpl.cpp:84-150 does.  Host arrays. */
int mpid_set_multipoles(mpid_context* ctx, const double* charge, const double* dipole, const double* quadrupole,
                        const double* octopole, const int* axis_type, const int* atom_z, const int* atom_x,
                        const int* atom_y, const double* thole, const double* polarity);

/* Covalent maps (MPIDForce::setCovalentMap, MPIDForce.h:291-308) as CSR over (atom, type):
 * offsets has 8*num_atoms+1 entries, type order Covalent12..15, PolarizationCovalent11..14. */
int mpid_set_covalent(mpid_context* ctx, const int* offsets, const int* index);

/* Evaluate with host buffers (CalcMPIDForceKernel::execute, mpidKernels.h:77).
 * positions: 3n; box: 9, the rows a, b, c of the periodic box in OpenMM's reduced form
 * (a = (ax, 0, 0), b = (bx, by, 0), c = (cx, cy, cz), |bx|, |cx| <= ax/2, |cy| <= by/2;
 * rectangular or triclinic; MPIDReferenceForce.cpp:2620-2675); forces: 3n, ADDED to;
 * energy: returns the energy (may be NULL). */
int mpid_evaluate(mpid_context* ctx, const double* positions, const double* box, double* forces, double* energy);

/* Same with device pointers on `stream` (cudaStream_t, may be NULL for the legacy stream).
 * d_forces is added to; d_energy (1 double) is overwritten.  Returns after enqueueing only
 * when the mutual solver's convergence allows; results are ready when the stream is. */
int mpid_evaluate_device(mpid_context* ctx, const double* d_positions, const double* box, double* d_forces,
                         double* d_energy, void* stream);

/* mpid_evaluate_device without any allocation.  No reference counterpart: the reference
 * kernel runs inside OpenMM, which owns all memory.  For callers that may not allocate
 * device memory while they evaluate: integrators that reserve a fixed device-memory
 * budget up front and must not exceed it mid-run, and hosts whose own allocator holds
 * the device memory (a framework's caching allocator or a plugin host that forbids
 * foreign cudaMalloc calls, which would otherwise fail or fragment its pool).  The
 * ordinary call allocates only when its neighbour lists must grow; this one keeps the
 * neighbour lists and the pair kernel's per-task energies in one static 8 MiB device
 * array per device and never grows anything (mpid_stats.device_allocations does not
 * change across it).
 *  - PME only.  Size limit: npad x (longest neighbour list rounded up to 32) <= 1,835,008
 *    entries (npad = atoms rounded up to 32), e.g. about 5,000 water atoms at a 0.9 nm
 *    cutoff.  Larger systems, and systems whose tile lists have not been sized by one
 *    mpid_evaluate_device call, are rejected with MPID_ERR_INVALID before anything is
 *    written to d_forces; the context stays usable.
 *  - Nothing in the array needs to start at zero: each call writes the lists and clears
 *    the energy partials before using them.
 *  - The first call on a device looks the array up (cudaGetSymbolAddress); make that
 *    first call before any stream capture.
 *  - The array is shared by every context of the process on that device: calls must not
 *    overlap in time on a device, from any thread or stream, or they race on it.
 *  - The caller's current device is left as it was.
 * Arguments and results as mpid_evaluate_device; the getters and gradient calls that
 * follow work as after mpid_evaluate_device (the gradient calls rebuild the context's own
 * neighbour lists before they read them). */
int mpid_evaluate_device_noalloc(mpid_context* ctx, const double* d_positions, const double* box, double* d_forces,
                                 double* d_energy, void* stream);

/* Dipoles of the last evaluation in caller order, 3n host doubles (e nm):
 * which 0 induced (getInducedDipoles), 1 lab-frame permanent (getLabFramePermanentDipoles),
 * 2 total (getTotalDipoles); mpidKernels.h:79-81.  which 3 returns the permanent
 * electric field at each atom (e/nm^2, before multiplication by the polarisability). */
int mpid_get_dipoles(mpid_context* ctx, int which, double* out);

/* System multipole moments at `positions` (CalcMPIDForceKernel::getSystemMultipoleMoments,
 * mpidKernels.h:86; MPIDReferenceForce.cpp:2349-2462): induced dipoles are solved at these
 * positions, positions are taken relative to the centre of `masses` (n doubles), and out
 * receives 13 values: charge (e), dipole x y z (Debye), quadrupole xx xy xz yx yy yz zx zy
 * zz (Debye-A, traceless, including the atoms' own quadrupoles). */
int mpid_get_system_multipole_moments(mpid_context* ctx, const double* positions, const double* box,
                                      const double* masses, double* out);

/* Electrostatic potential (kJ/mol/e) at ngrid points (3 doubles each), with the induced
 * dipoles solved at `positions` (CalcMPIDForceKernel::getElectrostaticPotential,
 * mpidKernels.h:83-84; MPIDReferenceForce.cpp:2464-2528): bare Coulomb potential of each
 * atom's charge, permanent + induced dipole and quadrupole, minimum-imaged under PME. */
int mpid_get_electrostatic_potential(mpid_context* ctx, const double* positions, const double* box,
                                     const double* grid, int ngrid, double* out);

/* Gradient of the energy at `positions` with respect to every atom's molecular-frame
 * multipole parameters, 20 doubles per atom in caller order: charge, dipole X Y Z,
 * quadrupole XX XY YY XZ YZ ZZ, octopole XXX XXY XYY YYY XXZ XYZ YYZ XZZ YZZ ZZZ (the
 * component orders of MPIDForce::addMultipole), kJ/mol per parameter unit.  Each
 * component is the partial derivative with the other components held fixed.  No
 * reference counterpart: the reference has no parameter derivatives.  Uses the
 * stationarity of the induced dipoles, so no extra linear solve is needed. */
int mpid_get_parameter_gradients(mpid_context* ctx, const double* positions, const double* box, double* out);

/* One evaluation at `positions` returning any of: forces (3n, ADDED to, as
 * mpid_evaluate), the energy, the multipole-parameter gradients (20n, as
 * mpid_get_parameter_gradients) and the polarisation-parameter gradients (4n per atom:
 * dE/d(molecular-frame polarisability X Y Z) in kJ/mol/nm^3 and dE/d(Thole width) in
 * kJ/mol).  Each pointer may be NULL.  Mutual and Direct use the stationarity of the
 * induced dipoles; Extrapolated adds the explicit adjoint sums over its perturbation
 * orders.  A polarisability of 0 gets a gradient of 0 (Mutual, Direct).  No reference
 * counterpart: the fitting entry point of this library. */
int mpid_evaluate_with_gradients(mpid_context* ctx, const double* positions, const double* box, double* forces,
                                 double* energy, double* multipole_grad, double* polarization_grad);

/* Evaluate `count` independent contexts (PME, one device) at once: for each k, energy
 * (energies[k]), forces ADDED to forces[k] (3n; forces or forces[k] may be NULL) and,
 * where multipole_grad / polarization_grad and their k-th pointer are non-NULL, the
 * gradients of mpid_evaluate_with_gradients.  Host arrays.  No reference counterpart:
 * the batched entry point of this library (parameter fitting over many small boxes).
 * Each context's evaluation runs with no host synchronisation -- list shape and
 * mutual-solver length taken from its previous evaluation -- in one of three launch modes:
 *   launch_mode 0 (fused): one launch per operation for all boxes.  Every box's evaluation
 *     is recorded as a sequence of operations, and operation i of all boxes becomes one
 *     kernel launch over the blocks of every box (each block runs its own box's
 *     parameters), or one batched cuFFT transform per grid size; the sequence is captured
 *     as one CUDA graph and replayed while no box changes shape.  Boxes of at most 4096
 *     atoms that all request the same gradients and evaluate the same way (precision,
 *     polarisation type, covalently scaled pairs present or not); otherwise the call
 *     fails with MPID_ERR_INVALID and launch_mode k > 0 takes the batch.
 *   launch_mode -1: each box's evaluation is a graph of its own; the graphs of all boxes
 *     run as one launch of a parent graph.
 *   launch_mode k > 0: each box's graph is launched on one of k streams.
 * After the launch each context's list sizes, solver convergence and FP64 residual are
 * checked; a context that fails a check (or is evaluated for the first time) gets the
 * ordinary evaluation instead, so the results are those of mpid_evaluate_with_gradients.
 * type_grad: NULL, or [ntypes][24] per-type gradient sums over all boxes (see
 * mpid_set_atom_types); per-atom gradients are then returned only where requested.
 * Calls are serialised within the process; a context may appear once per call. */
int mpid_evaluate_batch(mpid_context* const* ctxs, int count, const double* const* positions, const double* const* boxes,
                        double* const* forces, double* energies, double* const* multipole_grad,
                        double* const* polarization_grad, double* type_grad, int launch_mode);

/* Parameter types of the atoms (original order, 0 .. ntypes-1, ntypes <= 16; ntypes 0
 * clears them) for the per-type gradient sums of mpid_evaluate_batch: with type_grad
 * non-NULL the batch computes both gradient passes of every box and writes
 * type_grad[t][24] = the sum over the atoms of type t of all boxes of the 20 multipole and
 * 4 polarisation gradient components (the layout of multipole_grad and polarization_grad
 * side by side), summed on the device per box and then over the boxes in order.  No
 * reference counterpart (parameter fitting). */
int mpid_set_atom_types(mpid_context* ctx, const int* types, int ntypes);

/* Launch configuration: the largest number of sub-ranges each pair-kernel work item
 * (32 atoms x 32 list entries) is cut into, one warp each -- a power of two up to 32, or
 * 0 for the automatic choice, which cuts until a launch holds two waves of warps of the
 * whole GPU.  Contexts evaluated together (mpid_evaluate_batch, host threads) share the
 * GPU, where fewer, longer warps can be faster; the fitting module's autotuner picks the
 * bound by timing.  Results differ only in the rounding of the FP32 partial sums.  No
 * reference counterpart. */
int mpid_set_work_split(mpid_context* ctx, int max_split);

/* PME parameters in use (CalcMPIDForceKernel::getPMEParameters, mpidKernels.h:103). */
int mpid_get_pme_parameters(mpid_context* ctx, double* alpha, int* nx, int* ny, int* nz);

int mpid_get_stats(mpid_context* ctx, mpid_stats* out);

/* Message of the last failure on this thread ("" if none). */
const char* mpid_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
