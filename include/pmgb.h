/*
 * pmgb.h - C ABI of the GB300-native PM / P3M force-and-step path.
 *
 * Plain C: handles, plain pointers and sizes, int status codes; no C++ or torch types.  Every
 * entry point replaces one piece of the reference's PMMethod / PMMethodGPU / P3MMethod /
 * ChainingMesh call surface (paths below are within the reference project); the C++ facade in
 * include/pmgb/ and the Python mirror in particlesimulation_gb300/ sit on top of it.
 *
 * Units.  Inputs are in the caller's "original" units, as the reference's constructors take
 * them.  Inside a handle everything is kept in the reference's code units (x/H, v*DT/H,
 * a*DT^2/H, m*4*pi*G*DT^2/H^3; include/unitConversions.h:8-50).  Getters take a `units`
 * argument.
 *
 * Threading.  Each handle owns one CUDA stream and all of its device memory.  Handles are
 * independent; calls on one handle are not thread-safe.  No call throws; failures return a
 * status and pmgb_last_error() describes the last one.
 */
#ifndef PMGB_H
#define PMGB_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define PMGB_OK 0
#define PMGB_EINVAL 1   /* bad argument (reference: std::invalid_argument) */
#define PMGB_ECUDA 2    /* a CUDA call failed */
#define PMGB_EESCAPED 3 /* a particle left the computational box; the run stopped there */
#define PMGB_ETIMEOUT 4 /* a bounded device wait gave up */
#define PMGB_ENOMEM 5   /* device allocation failed */

/* ---- enums: same names order and values as the reference ---- */
/* InterpolationScheme (include/pmConfig.h:3) */
#define PMGB_NGP 0
#define PMGB_CIC 1
#define PMGB_TSC 2
/* FiniteDiffScheme (include/pmConfig.h:4) */
#define PMGB_TWO_POINT 0
#define PMGB_FOUR_POINT 1
/* GreensFunction (include/pmConfig.h:5) */
#define PMGB_DISCRETE_LAPLACIAN 0
#define PMGB_S1_OPTIMAL 1
#define PMGB_S2_OPTIMAL 2
#define PMGB_POOR_MAN 3
/* CloudShape (include/greensFunctions.h:7) */
#define PMGB_S1 0
#define PMGB_S2 1
/* units of getters */
#define PMGB_UNITS_CODE 0
#define PMGB_UNITS_ORIGINAL 1
/* external field kinds: the reference passes a std::function (include/pmMethod.h:17); on the
 * device it is an enum with parameters.  SPH_RAD_DECR = sphRadDecrField(pos, center, R, M, G)
 * (source/externalFields.cpp:4-15). */
#define PMGB_EXT_NONE 0
#define PMGB_EXT_SPH_RAD_DECR 1

typedef struct pmgb_external_field {
  int kind;
  float center[3];
  float R, M, G;
} pmgb_external_field;

/* Arguments of PMMethod(state, masses, effectiveBoxSize, externalField, externalPotential,
 * H, DT, G, is, fds, gFunc, particleDiameter, grid) (include/pmMethod.h:14-26) with the grid
 * given by its point counts, as PMMethodGPU takes it (include_gpu/PMMethodGPU.h:14-27). */
typedef struct pmgb_pm_config {
  int grid[3];          /* gridPoints (x, y, z), each in [4, 4096]; meshes whose sides are all
                           powers of two in [8, 512] take the specialised Poisson solve, others a
                           mixed-radix one (any factors, as the reference's FFT plug-ins) */
  float box[3];         /* effectiveBoxSize, original units */
  float H, DT, G;
  int interpolation;    /* PMGB_NGP / PMGB_CIC / PMGB_TSC */
  int finite_diff;      /* PMGB_TWO_POINT / PMGB_FOUR_POINT */
  int greens;           /* PMGB_DISCRETE_LAPLACIAN / ... */
  float particle_diameter; /* original units */
  pmgb_external_field ext;
  /* PM-only runs re-sort particles every `sort_interval` steps (results do not depend on the
   * order; only locality does).  0 = default (16). */
  int sort_interval;
  /* 0: the reference's isolated setup (particles must stay in [0, box]; leaving it stops a
   * run, PMGB_EESCAPED).  1: periodic box equal to the mesh: positions wrap after each drift and
   * there is no escape test (the reference has no periodic mode; mesh indices always wrap). */
  int periodic;
} pmgb_pm_config;

/* Arguments of P3MMethod(pm, compBoxSize, cutoffRadius, particleDiameter, H, softeningLength,
 * cloudShape, useSRForceTable, enableYSorting) (include/p3mMethod.h:13-26). */
typedef struct pmgb_p3m_config {
  float comp_box[3];   /* compBoxSize, original units */
  float cutoff;        /* cutoffRadius, original units */
  float particle_diameter;
  float softening;     /* softeningLength */
  int cloud_shape;     /* PMGB_S1 / PMGB_S2 */
  int use_table;       /* useSRForceTable (1 = 500-entry table, 0 = direct formula) */
  int y_sorting;       /* enableYSorting: cell lists ordered by y (ties by index) or by
                          descending index, exactly as ChainingMesh::fillWithYSorting / fill */
} pmgb_p3m_config;

typedef struct pmgb_pm pmgb_pm;   /* PMMethod / PMMethodGPU */
typedef struct pmgb_p3m pmgb_p3m; /* P3MMethod (borrows a pmgb_pm) */

/* ---------------------------------------------------------------- PM ---------------- */

/* PMMethodGPU::PMMethodGPU (source/PMMethodGPU.cu:32-68): copies state (n positions then n
 * velocities, xyz triplets, original units) and masses to the device, converting to code units.
 * Precomputes the influence function (initGreensFunction, source/pmMethod.cpp:164-185) in FP64
 * on the device. */
int pmgb_pm_create(const pmgb_pm_config* cfg, int n, const float* state, const float* masses,
                   pmgb_pm** out);
/* ~PMMethodGPU (source/PMMethodGPU.cu:70-73). */
int pmgb_pm_destroy(pmgb_pm* pm);

/* PMMethod::initGreensFunction (source/pmMethod.cpp:164-185); also done by create. */
int pmgb_pm_init_greens_function(pmgb_pm* pm);

/* PMMethod::pmMethodStep (source/pmMethod.cpp:137-144): accelerations at the current
 * positions (deposit, FFT, influence function, inverse FFT, finite-difference field,
 * interpolation, external field).  No kick, no drift. */
int pmgb_pm_method_step(pmgb_pm* pm);

/* PMMethod::run (source/pmMethod.cpp:62-135) without recorder or diagnostics: initial force,
 * half kick, then sim_length + 1 drift / force / kick iterations, stopping on an escaped
 * particle exactly where the reference breaks.  Returns PMGB_EESCAPED in that case and
 * *steps_done = completed iterations. */
int pmgb_pm_run(pmgb_pm* pm, int sim_length, int* steps_done);

/* The body of PMMethod::run's loop (source/pmMethod.cpp:79-122: drift, force, kick) repeated
 * n_steps times, continuing from the state run() or a previous advance left (positions at an
 * integer step, velocities half a step ahead).  Stops on an escaped particle like run().
 * *device_ms (may be NULL) receives the device time of the whole call, measured with CUDA
 * events on the handle's stream. */
int pmgb_pm_advance(pmgb_pm* pm, int n_steps, int* steps_done, float* device_ms);

/* PMMethod::getParticles (include/pmMethod.h:33): positions, velocities (half-step, as the
 * reference stores them) and accelerations of the particles in their original index order.
 * Any pointer may be NULL.  units = PMGB_UNITS_CODE or PMGB_UNITS_ORIGINAL (accelerations are
 * converted with accelerationToOriginalUnits). */
int pmgb_pm_get_particles(pmgb_pm* pm, float* pos, float* vel, float* acc, int units);

/* PMMethodGPU::copyParticlesHostToDevice (include_gpu/PMMethodGPU.h:47): replace positions and
 * velocities (original index order, `units`) of all particles. */
int pmgb_pm_set_particles(pmgb_pm* pm, const float* pos, const float* vel, int units);

/* PMMethod::escapedComputationalBox (source/pmMethod.cpp:146-156), on the device. */
int pmgb_pm_escaped(pmgb_pm* pm, int* escaped);

/* PMMethodGPU::copyGridDensityToHost / copyGridPotentialToHost + getGridDensity /
 * getGridPotential (include_gpu/PMMethodGPU.h:48-55): the last step's density and potential
 * meshes, nx*ny*nz floats, x fastest, code units. */
int pmgb_pm_get_density(pmgb_pm* pm, float* density);
int pmgb_pm_get_potential(pmgb_pm* pm, float* potential);
/* The influence function as applied: (nx/2+1)*ny*nz floats (x fastest), already symmetrised
 * over k and -k and divided by nx*ny*nz (the inverse FFT's 1/N, folded in). */
int pmgb_pm_get_greens_function(pmgb_pm* pm, float* ghat);

/* Device time of each stage of the last pmgb_pm_method_step / p3m force, in milliseconds:
 * [sort, deposit, fft_forward+green+inverse, interpolation, pair pass]. */
int pmgb_pm_stage_times(pmgb_pm* pm, float* ms5);

/* Number of particles and the grid of a handle. */
int pmgb_pm_size(pmgb_pm* pm, int* n, int* grid3);

/* The handle's CUDA stream (a cudaStream_t), on which every call of the handle and of the P3M /
 * closure handles over it enqueues its work; for callers that time or order their own work
 * against it.  No reference counterpart (the reference's GPU path uses the default stream). */
int pmgb_pm_get_stream(pmgb_pm* pm, void** stream);

/* ---------------------------------------------------------------- stepper ----------- */
/* The leapfrog free functions of source/leapfrog.cpp:5-24 (include/leapfrog.h:6-12), in the
 * reference's float arithmetic: */
#define PMGB_LEAPFROG_HALF_KICK 0    /* setHalfStepVelocities:    v += 0.5 dt a */
#define PMGB_LEAPFROG_DRIFT 1        /* updatePositions:          x += dt v */
#define PMGB_LEAPFROG_KICK 2         /* updateVelocities:         v += dt a */
#define PMGB_LEAPFROG_INTEGER_STEP 3 /* setIntegerStepVelocities: u = v + 0.5 dt a */
/* On host arrays of n xyz triplets (the reference's std::vector<Particle> argument), computed on
 * the device: pos is written by DRIFT, vel by the kicks, int_vel by INTEGER_STEP; arrays an
 * operation does not use may be NULL. */
int pmgb_leapfrog(int op, int n, float* pos, float* vel, const float* acc, float* int_vel, float dt);
/* On a PM handle's particles on the device, code units (the reference's run loop calls them with
 * dt = 1 in code units), with the accelerations of the handle's last force evaluation;
 * INTEGER_STEP keeps u in the handle (read with pmgb_pm_get_integer_step_velocities). */
int pmgb_pm_leapfrog(pmgb_pm* pm, int op, float dt);
/* Particle::integerStepVelocity (include/particle.h:10) of every particle (original order) as
 * the last PMGB_LEAPFROG_INTEGER_STEP set it (zero before), `units`. */
int pmgb_pm_get_integer_step_velocities(pmgb_pm* pm, float* vel, int units);
/* PMMethod::totalExternalForceOrigUnits (source/pmMethod.cpp:158-162): sum over particles of
 * m g(x) in original units (zero without an external field); summed in double on the device. */
int pmgb_pm_total_external_force(pmgb_pm* pm, float* force3);

/* ---------------------------------------------------------------- run diagnostics ---- */

/* What PMMethod::run / P3MMethod::run(..., collectDiagnostics = true) record once per loop
 * iteration, right after its drift (source/pmMethod.cpp:66-106, source/p3mMethod.cpp:69-130,
 * source/PMMethodGPU.cu:86-139): the SimInfo quantities of source/simInfo.cpp:50-127, in
 * original units, summed in double on the device.  One record = PMGB_DIAG_WIDTH doubles: */
#define PMGB_DIAG_WIDTH 12
#define PMGB_DIAG_POTENTIAL 0          /* potentialEnergy(density, potential, ...): 0.5 H^3
                                          sum(rho phi) over the mesh + sum(m Phi_ext(x)) */
#define PMGB_DIAG_KINETIC 1            /* kineticEnergy: sum(0.5 m |v|^2), half-step v */
#define PMGB_DIAG_MOMENTUM 2           /* totalMomentum: sum(m u), u = v + a/2 (3 values) */
#define PMGB_DIAG_ANGULAR_MOMENTUM 5   /* totalAngularMomentum: sum(m x cross u) (3) */
#define PMGB_DIAG_EXPECTED_MOMENTUM 8  /* initial momentum + DT sum(totalExternalForce) (3) */
#define PMGB_DIAG_EXTERNAL_POTENTIAL 11 /* the sum(m Phi_ext(x)) part of PMGB_DIAG_POTENTIAL */

/* capacity > 0: record diagnostics during pmgb_pm_run / pmgb_p3m_run / pmgb_pm_advance, keeping
 * the first `capacity` records (device memory: capacity * 96 bytes plus 4 bytes per mesh cell
 * for the density copy).  Clears the records and sets the expected momentum to the current
 * total momentum (SimInfo::setInitialMomentum); pmgb_pm_run does both again when it starts.
 * With diagnostics on, every iteration also rounds the masses through original units and back
 * as the reference does (massToOriginalUnits / massToCodeUnits).  capacity = 0: off. */
int pmgb_pm_set_diagnostics(pmgb_pm* pm, int capacity);

/* Copies min(records taken, capacity, max_records) records into `records` (row-major,
 * PMGB_DIAG_WIDTH doubles each) and sets *count = records taken since they were last cleared
 * (records beyond the capacity are dropped).  *count = 0 when diagnostics are off. */
int pmgb_pm_get_diagnostics(pmgb_pm* pm, double* records, int max_records, int* count);

/* ---------------------------------------------------------------- samplers ----------- */

/* PlummerSampler(seed).sample(center, a, rMax, M, G, n) (source/plummerSampler.cpp:11-83; the
 * argument order of its definition, which the reference's callers use) and
 * DiskSamplerLinear(seed).sample(center, rb, mb, rd, md, thickness, G, n, r0)
 * (source/diskSamplerLinear.cpp:10-74), on the device, one thread per particle, drawing the
 * reference's own random stream (std::default_random_engine(seed), i.e. minstd_rand0, through
 * uniform_real_distribution<float>).  offset = numbers already drawn from that engine (6 per
 * Plummer particle, 3 per disk particle of earlier sample() calls on the same sampler).
 * state = 6n floats (host): n positions then n velocities. */
int pmgb_sample_plummer(unsigned int seed, unsigned long long offset, const float* center, float a,
                        float r_max, float M, float G, int n, float* state);
int pmgb_sample_disk_linear(unsigned int seed, unsigned long long offset, const float* center,
                            float rb, float mb, float rd, float md, float thickness, float G, int n,
                            float r0, float* state);

/* ---------------------------------------------------------------- StateRecorder ------ */

/* StateRecorder(particlesCnt, framesCnt, outputDirPath, positionsFile, energyFile,
 * momentumFile, expectedMomentumFile, angularMomentumFile, fieldFile)
 * (source/stateRecorder.cpp:5-44): creates output_dir, writes the int32 (n, frames) headers
 * of the binary files.  names = the six file names in that order (positions, energy, momentum,
 * expected momentum, angular momentum, field); NULL = the reference's defaults, an empty name
 * = that output left out.  with_field reserves device room for field frames.  Frames are
 * packed on the device and written by a host thread from pinned buffers as they fill. */
typedef struct pmgb_recorder pmgb_recorder;
int pmgb_recorder_create(int n, int frames, const char* output_dir, const char* const* names,
                         int with_field, pmgb_recorder** out);
int pmgb_recorder_destroy(pmgb_recorder* rec);

/* StateRecorder::flush (source/stateRecorder.cpp:109-119): waits for the frames in flight,
 * writes the text files; copies the output directory into dir_out (may be NULL). */
int pmgb_recorder_flush(pmgb_recorder* rec, char* dir_out, int cap);

/* Frames written to the binary files so far (after waiting for those in flight). */
int pmgb_recorder_frames_written(pmgb_recorder* rec, long long* frames);

/* PMMethod::run(stateRecorder, simLength, collectDiagnostics, recordField) and
 * P3MMethod::run (source/pmMethod.cpp:62-135, source/p3mMethod.cpp:59-166): the run of
 * pmgb_pm_run recording every iteration's positions (recordPositions), with record_field the
 * acceleration of the iteration (recordField), with collect_diagnostics the energy and momentum
 * lines (run diagnostics turned on with room for the run if needed); flushes the recorder at the
 * end.  Returns like pmgb_pm_run. */
int pmgb_pm_run_recorded(pmgb_pm* pm, pmgb_recorder* rec, int sim_length, int collect_diagnostics,
                         int record_field, int* steps_done);

/* ---------------------------------------------------------------- P3M --------------- */

/* P3MMethod::P3MMethod (source/p3mMethod.cpp:19-48): chaining mesh and short-range force
 * table.  Borrows `pm` (which must outlive the P3M handle) and adds the short-range pair pass
 * to every force evaluation of that PM handle while it exists. */
int pmgb_p3m_create(pmgb_pm* pm, const pmgb_p3m_config* cfg, pmgb_p3m** out);
int pmgb_p3m_destroy(pmgb_p3m* p3m);

/* One P3M force evaluation: pmMethodStep + calculateShortRangeForces + correctAccelerations
 * (source/p3mMethod.cpp:63-73, 168-192, 50-57).  No kick, no drift. */
int pmgb_p3m_force(pmgb_p3m* p3m);

/* P3MMethod::run (source/p3mMethod.cpp:59-166) without recorder or diagnostics. */
int pmgb_p3m_run(pmgb_p3m* p3m, int sim_length, int* steps_done);

/* ChainingMesh cell lists of the last force evaluation (source/chainingMesh.cpp:20-58):
 * order[] = particle ids cell after cell (cell index x + y*Mx + z*Mx*My), counts[] = list
 * length per cell (Mx*My*Mz ints).  dims may be queried alone (order = counts = NULL). */
int pmgb_p3m_get_cell_lists(pmgb_p3m* p3m, int* order, int* counts, int* dims3);

/* The 500-entry short-range force table (initSRForceTable, source/p3mMethod.cpp:275-294) and
 * its r^2 spacing, code units. */
int pmgb_p3m_get_sr_table(pmgb_p3m* p3m, float* table500, float* delta_sq);

/* Ordered particle pairs (i, j), i != j, closer than the cutoff in the last force evaluation
 * (each unordered pair counts twice).  No reference counterpart: it sizes the pair pass's
 * FLOP count (20 FLOP per unordered pair). */
int pmgb_p3m_pair_count(pmgb_p3m* p3m, unsigned long long* ordered_pairs);
/* Turns the in-range pair counter of force evaluations on or off (off by default; counting
 * costs a few percent of the pair pass). */
int pmgb_p3m_set_pair_counting(pmgb_p3m* p3m, int enable);
/* Each pair once, as the reference's half-shell pass (source/p3mMethod.cpp:247-273, 296-322)
 * does: with y-sorted lists and equal masses the pair pass evaluates the dense sub-column pairs
 * below a cost bound (each taken whole by one warp or CTA) once, writing both particles' partial
 * forces to slots of their own, and the rest from both sides.  On by default where it applies (its
 * slots take 27 s^2 x 16 B per particle, s the sub-columns per cell axis: 3.9, 6.9 or 10.8 KB at
 * s = 3, 4, 5; allocated with the handle when that is at most a quarter of the free device memory;
 * otherwise the handle stays one-sided and enable has no effect); off evaluates every pair from
 * both sides.  Both are deterministic; they differ by float rounding.  units_last_pass
 * (may be NULL): the sub-column pairs the last force evaluation took once (0 when it ran
 * one-sided).  No reference counterpart (a switch of this implementation). */
int pmgb_p3m_set_symmetric(pmgb_p3m* p3m, int enable);
int pmgb_p3m_get_symmetric(pmgb_p3m* p3m, int* enabled, unsigned int* units_last_pass);
/* Sub-columns per cell axis the pair pass splits each chaining-mesh cell into (x and z): 1 for
 * the reference's unsorted lists; with y-sorted lists 5 where the handle's particles average at
 * least 96 per cell (N >= 96 Mx My Mz), 4 from 32, else 3, lowered (not below 3) until the
 * symmetric slots fit a quarter of the free device memory.  Fixed at creation.  The cell lists
 * handed out (pmgb_p3m_get_cell_lists) are whole cells either way.  No reference counterpart. */
int pmgb_p3m_get_subcolumns(const pmgb_p3m* p3m, int* per_axis);

/* ---------------------------------------------------------------- ensemble ----------- */
/* No counterpart in the reference (one system per process there).  n_systems independent PM
 * systems, each exactly a pmgb_pm (cfgs[s], counts[s] particles, states[s] = positions then
 * velocities, masses[s]), advanced together: every stage of a step is one launch over all
 * systems (persistent kernels over a table of systems and work items), each step one CUDA
 * graph.  All systems share the interpolation and difference schemes; meshes, particle
 * counts, boxes, Green's functions and external fields may differ.  Tile shapes are picked at
 * creation by timing candidates (they do not change results: each system is bit-identical to
 * the same system run by a pmgb_pm handle). */
typedef struct pmgb_ensemble pmgb_ensemble;
int pmgb_ensemble_create(int n_systems, const pmgb_pm_config* cfgs, const int* counts,
                         const float* const* states, const float* const* masses,
                         pmgb_ensemble** out);
int pmgb_ensemble_destroy(pmgb_ensemble* e);
/* PMMethod::run for every system (escaped[s] = 1 where system s stopped on an escape). */
int pmgb_ensemble_run(pmgb_ensemble* e, int sim_length, int* escaped, float* device_ms);
/* n_steps more loop iterations of every system, continuing from run(). */
int pmgb_ensemble_advance(pmgb_ensemble* e, int n_steps, float* device_ms);
int pmgb_ensemble_get_particles(pmgb_ensemble* e, int system, float* pos, float* vel, float* acc,
                                int units);
/* Autotuner choices: particles per deposit thread, x-pass rows per CTA (0: half, 1: default,
 * 2: double the default), and the six candidate timings in ms. */
int pmgb_ensemble_tuning(pmgb_ensemble* e, int* deposit_ppt, int* x_rows_mult, float* timings6);
int pmgb_ensemble_size(pmgb_ensemble* e, int* n_systems, long long* total_particles);

/* ---------------------------------------------------------------- learned closure ---- */
/* No counterpart in the reference.  A plain P3M pair pass at cutoff re is replaced by one at a
 * reduced cutoff re' plus an MLP that predicts the missing short-range force of the pairs at
 * re' <= r < re from the 4x4x4 patch of cell masses of the reduced chaining mesh around each
 * particle and its in-cell offset (67 inputs, 3 hidden GELU layers of 64, BF16 weights, FP32
 * accumulation, tensor-core kernels).  It is trained on the GPU on residuals the plain P3M
 * itself produces; the plain P3M judges it and is the fallback.  Modes: */
#define PMGB_CLOSURE_FULL 0         /* plain P3M at the full cutoff */
#define PMGB_CLOSURE_LEARNED 1      /* reduced-cutoff pair pass + learned residual */
#define PMGB_CLOSURE_REDUCED_ONLY 2 /* reduced-cutoff pair pass alone (what the MLP adds to) */

typedef struct pmgb_closure pmgb_closure;

/* Creates the full- and reduced-cutoff pair passes over `pm` (which must have no P3M handle;
 * destroy the closure before the PM handle), `capacity` training rows, parameters initialised
 * from `seed`.  Starts in PMGB_CLOSURE_FULL. */
int pmgb_closure_create(pmgb_pm* pm, const pmgb_p3m_config* full_cfg, float reduced_cutoff,
                        int capacity, unsigned long long seed, pmgb_closure** out);
int pmgb_closure_destroy(pmgb_closure* c);
int pmgb_closure_set_mode(pmgb_closure* c, int mode);
int pmgb_closure_get_mode(pmgb_closure* c, int* mode);
/* Adds (features, residual) rows for every `stride`-th particle at the current positions:
 * residual = full-cutoff minus reduced-cutoff P3M acceleration.  *total = rows collected. */
int pmgb_closure_collect(pmgb_closure* c, int stride, int* total);
/* Adam on the collected rows (mean squared error, cosine learning-rate decay). */
int pmgb_closure_train(pmgb_closure* c, int epochs, int batch, float lr, float* final_loss);
int pmgb_closure_param_count(void);
int pmgb_closure_get_params(pmgb_closure* c, float* params, int count);
int pmgb_closure_set_params(pmgb_closure* c, const float* params, int count);
/* Median relative difference between the learned and the full-cutoff P3M accelerations at the
 * current positions, over the particles of every `stride`-th slice (64 particles of a chaining-
 * mesh sub-column) of the full-cutoff pair pass, which then covers only those slices (about
 * 1/stride of its cost); with the table-free formula and softening, over every `stride`-th
 * particle by index (full pass).  The learned force is the last step's when that step was
 * learned and the particles have not moved since. */
int pmgb_closure_judge(pmgb_closure* c, int stride, float* median_rel_err);
/* n_steps run-loop iterations in the current mode.  In PMGB_CLOSURE_LEARNED every
 * judge_interval-th step (0, judge_interval, ...) is judged after it ran, at the positions it
 * drifted to (pmgb_closure_judge on the learned force it used); a median error above `bound` has
 * the step taken again from its start with plain P3M, and the rest of the run too
 * (*fallback_step = that step, else -1), so no step keeps a rejected force.  The step's start
 * state is kept in 32 bytes per particle of device memory, allocated on the first judged run.
 * device_ms counts both attempts of a rejected step. */
int pmgb_closure_run(pmgb_closure* c, int n_steps, float bound, int judge_interval,
                     int judge_stride, int* steps_done, int* fallback_step, float* device_ms);
/* Test support: the 67 inputs of every particle (original order) and its patch mass; the
 * output scale c and the reduced mesh dimensions. */
int pmgb_closure_features(pmgb_closure* c, float* x, float* spatch);
int pmgb_closure_scales(pmgb_closure* c, float* out_scale, int* dims3);
/* Test support: the MLP kernels on host data.  params: pmgb_closure_param_count() floats
 * (W1 64x80, b1, W2 64x64, b2, W3 64x64, b3, W4 8x64, b4 8; padding zero).  x: n x 67,
 * y: n x 3, t: n x 3 targets; gradients of the mean over rows of |y - t|^2. */
int pmgb_mlp_eval(const float* params, int n, const float* x, float* y);
int pmgb_mlp_gradients(const float* params, int n, const float* x, const float* t, float* grad,
                       float* loss);
/* Test support: the bounded mbarrier wait of the tensor-core kernels, on a barrier that gets its
 * one arrival (arrive = 1: PMGB_OK) or none (arrive = 0: the wait gives up after `spins` tries
 * and the call returns PMGB_ETIMEOUT, the device context still usable). */
int pmgb_tc_wait_probe(int arrive, int spins);

/* Chaining-mesh cell lists built without allocating any device memory.  No counterpart in the
 * reference: it is for callers that cannot allocate device memory where they need the lists
 * (hosts that hand the library buffers from their own fixed pool, or step loops that must not
 * call cudaMalloc).  Same lists as pmgb_p3m_get_cell_lists: d_pos = n xyz triplets in code
 * units (device memory), d_order = n ints, d_counts = Mx*My*Mz ints (device memory), dims3 =
 * (Mx, My, Mz) on the host; cfg supplies comp_box, cutoff and y_sorting.  Runs on `stream`
 * (a cudaStream_t, NULL = default stream) without synchronising.  Limits: n <= 262,144 and
 * Mx*My*Mz <= 262,142; larger inputs return PMGB_EINVAL.  Its scratch (about 7.1 MiB) is a
 * fixed device array; under lazy module loading it is loaded on the first call on each device
 * (that call also looks its address up, so make it before any stream capture or any section
 * that must not allocate) and held until exit; calls that overlap on the GPU share the scratch
 * and race.  Particles outside the chaining mesh are not listed: d_order holds sum(counts)
 * entries and the rest of it is left as it was. */
int pmgb_chaining_mesh_fill_noalloc(const float* d_pos, int n, const pmgb_p3m_config* cfg,
                                    float H, int* d_order, int* d_counts, int* dims3,
                                    void* stream);

/* ---------------------------------------------------------------- FFT plug-in ------- */
/* FFTAdapter<float>::fft / ifft (include/FFTAdapter.h:6-15; FFTWAdapter, source/FFTWAdapter.cpp:
 * 27-43; KissFFTAdapter, include/kissFFTAdapter.h:16-29): 3D complex-to-complex transform of
 * nx*ny*nz complex values (interleaved re, im; x fastest, as the reference's Grid stores its
 * meshes), any lengths in [1, 8192].  Forward unnormalised; inverse = 1/(nx*ny*nz) times the
 * unnormalised inverse, as the reference's adapters scale.  in and out are host arrays of
 * 2*nx*ny*nz floats and may be the same array.  Mixed radix (4, 2, 3, 5, 7, other primes) on the
 * device. */
int pmgb_fft3d(int nx, int ny, int nz, const float* in, float* out, int inverse);

/* ---------------------------------------------------------------- direct sum -------- */
/* ppMethod's pairwise gravitational acceleration (source/ppMethod.cpp:23-36) restated in FP64
 * on the device, for the m targets idx[0..m) against all n particles: acc[3k..3k+2] =
 * sum_{j != idx[k]} -G m_j (x_i - x_j) / (|x_i - x_j|^2 + eps^2)^1.5.  pos = n xyz triplets and
 * masses (host, any consistent units); acc = m xyz triplets (host, double).  periodic_L > 0:
 * minimum-image separations in a cube of that side (no Ewald sum).  The yardstick of the force
 * error reports (the reference uses its PP integrator the same way in its accuracy scenarios,
 * source/demos.cpp:390-396, 617-621); deterministic (fixed summation order). */
int pmgb_direct_sum_fp64(int n, const float* pos, const float* masses, double G, double eps, int m,
                         const int* idx, double periodic_L, double* acc);

/* ---------------------------------------------------------------- misc -------------- */
/* FP32 FMA throughput of the current device in TFLOP/s, measured by a timed FMA kernel (the
 * roofline denominator of the FP32-bound pair pass).  No reference counterpart. */
int pmgb_fp32_peak_probe(float* tflops);
const char* pmgb_last_error(void);
/* Number of kernels this process has launched through the library. */
int pmgb_kernel_launches(long long* count);
/* Library build identification (architecture string). */
const char* pmgb_version(void);

#ifdef __cplusplus
}
#endif
#endif /* PMGB_H */
