/*
 * oracle_api.h - C interface of the CPU oracle (TEST INFRASTRUCTURE ONLY).
 *
 * Two libraries implement the functions declared here:
 *
 *   oracle/_ref/libpsref.so   "ref_*"  the reference's own CPU PMMethod / P3MMethod /
 *                                      ChainingMesh / ppMethod code, compiled from the
 *                                      reference sources by oracle/Makefile and driven by
 *                                      oracle/ref_shim.cpp.  Only buildable where the
 *                                      reference sources are present.
 *   oracle/_build/liboracle.so "port_*" oracle/port.cpp: a restatement of the same
 *                                      algorithms, templated on the scalar type, so the
 *                                      same code runs in float (mirrors the reference's
 *                                      FP32 arithmetic) and in double (the FP64 oracle).
 *
 * Nothing in the product (particlesimulation_gb300/, include/) links or calls these.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs use them, and
 * only as the reference results / the timed CPU baseline.
 *
 * Units follow the reference: inputs are in "original" units (state = N positions then N
 * velocities, each xyz float triplets); accelerations are returned in code units
 * (x/H, v*DT/H, a*DT^2/H, m*4*pi*G*DT^2/H^3), like Particle::acceleration after
 * PMMethod::pmMethodStep (reference source/pmMethod.cpp:62-75, include/unitConversions.h:8-50).
 */
#ifndef PSIM_ORACLE_API_H
#define PSIM_ORACLE_API_H

#ifdef __cplusplus
extern "C" {
#endif

/* Mirrors the PMMethod constructor arguments (reference include/pmMethod.h:14-26) plus the
 * grid size of Grid(gridPoints, ...) (include/grid.h:12).  Enum values equal the reference's
 * InterpolationScheme / FiniteDiffScheme / GreensFunction (include/pmConfig.h:3-5). */
typedef struct orc_pm_params {
  int nx, ny, nz;
  float box_x, box_y, box_z; /* effectiveBoxSize, original units */
  float H, DT, G;
  int is;  /* 0 NGP, 1 CIC, 2 TSC */
  int fds; /* 0 TWO_POINT, 1 FOUR_POINT */
  int gf;  /* 0 DISCRETE_LAPLACIAN, 1 S1_OPTIMAL, 2 S2_OPTIMAL, 3 POOR_MAN */
  float diameter; /* particleDiameter, original units */
  /* external field: 0 none, 1 sphRadDecrField(center, R, M, G) (source/externalFields.cpp:4-15) */
  int ext_kind;
  float ext_cx, ext_cy, ext_cz, ext_R, ext_M, ext_G;
  /* port only: 1 = wrap deposit / field indices periodically (the reference leaves them
   * unwrapped, which is only defined for particles away from the mesh edge). */
  int periodic;
} orc_pm_params;

/* Mirrors the P3MMethod constructor (include/p3mMethod.h:13-26). */
typedef struct orc_p3m_params {
  float comp_x, comp_y, comp_z; /* compBoxSize, original units */
  float cutoff;                 /* cutoffRadius, original units */
  float diameter;               /* particleDiameter, original units */
  float softening;              /* softeningLength, original units */
  int cloud_shape;              /* 0 S1, 1 S2 (include/greensFunctions.h:7) */
  int use_table;                /* useSRForceTable */
  int y_sorting;                /* enableYSorting */
} orc_p3m_params;

/* ---- reference (compiled from the reference sources) ---- */
int ref_pm_accel(const orc_pm_params* p, int n, const float* state, const float* masses,
                 float* acc, float* density, float* potential, float* green);
int ref_p3m_accel(const orc_pm_params* p, const orc_p3m_params* q, int n, const float* state,
                  const float* masses, float* acc);
/* run(recorder, sim_length, flags & 1, flags & 2) (collectDiagnostics, recordField; the last
 * argument holds the flags) with a StateRecorder writing into
 * outdir (positions.dat, energy.txt, momentum.txt, expected_momentum.txt,
 * angular_momentum.txt). */
int ref_pm_run(const orc_pm_params* p, int n, const float* state, const float* masses,
               int sim_length, const char* outdir, float* state_out, int* escaped,
               int collect_diagnostics);
int ref_p3m_run(const orc_pm_params* p, const orc_p3m_params* q, int n, const float* state,
                const float* masses, int sim_length, const char* outdir, float* state_out,
                int* escaped, int collect_diagnostics);
/* Chaining-mesh cell lists: order[] = particle ids cell by cell, counts[] = list length
 * per cell, dims[3] = (Mx, My, Mz).  pos_code = N xyz triplets in code units. */
int ref_chaining_mesh(const orc_p3m_params* q, float H, int n, const float* pos_code,
                      int y_sorting, int* order, int* counts, int* dims);
int ref_pp_accel(int n, const float* pos, const float* masses, float G, float eps, float* acc);
/* P3MMethod's FTable and deltaSquared (source/p3mMethod.cpp:42-47, 275-294). */
int ref_sr_table(const orc_p3m_params* q, float H, float* table /*500*/, float* delta_sq);
/* PlummerSampler(seed).sample(center, a, rMax, M, G, n) and DiskSamplerLinear(seed).sample(
 * center, rb, mb, rd, md, thickness, G, n, r0): 2n xyz triplets, positions then velocities. */
int ref_sample_plummer(unsigned int seed, const float* center, float a, float r_max, float M,
                       float G, int n, float* state_out);
int ref_sample_disk_linear(unsigned int seed, const float* center, float rb, float mb, float rd,
                           float md, float thickness, float G, int n, float r0, float* state_out);

/* ---- port (oracle/port.cpp); prec = 0 float, 1 double ---- */
int port_pm_accel(int prec, const orc_pm_params* p, int n, const float* state,
                  const float* masses, double* acc, double* density, double* potential,
                  double* green);
int port_p3m_accel(int prec, const orc_pm_params* p, const orc_p3m_params* q, int n,
                   const float* state, const float* masses, double* acc, double* acc_sr,
                   int nthreads);
/* Run loops.  diag != NULL turns on the reference's collectDiagnostics: one record of 12
 * doubles per loop iteration (layout of include/pmgb.h's PMGB_DIAG_*), at most diag_cap of
 * them stored; *diag_count = records taken. */
int port_pm_run(int prec, const orc_pm_params* p, int n, const float* state,
                const float* masses, int sim_length, double* state_out, int* escaped,
                double* diag, int diag_cap, int* diag_count);
int port_p3m_run(int prec, const orc_pm_params* p, const orc_p3m_params* q, int n,
                 const float* state, const float* masses, int sim_length, double* state_out,
                 int* escaped, int nthreads, double* diag, int diag_cap, int* diag_count);
int port_chaining_mesh(const orc_p3m_params* q, float H, int n, const float* pos_code,
                       int y_sorting, int* order, int* counts, int* dims);
/* FP64 direct sum (ppMethod.cpp:23-36 restated in double) for the targets idx[0..m):
 * acc[3*k..] = sum_j -G m_j (r_i - r_j) / (|r_i - r_j|^2 + eps^2)^1.5, pos in any
 * consistent units.  periodic_L > 0 applies the minimum-image convention. */
int port_pp_accel(int n, const double* pos, const double* masses, double G, double eps,
                  int m, const int* idx, double periodic_L, double* acc, int nthreads);
/* P3M accelerations (code units) of the targets idx[0..m): PM for all particles plus the
 * short-range sum over every particle within the cutoff, by brute force (no cell lists). */
int port_p3m_accel_targets(int prec, const orc_pm_params* p, const orc_p3m_params* q, int n,
                           const float* state, const float* masses, int m, const int* idx,
                           double* acc, int nthreads);
/* The SR force table of P3MMethod::initSRForceTable (p3mMethod.cpp:275-294), float. */
int port_sr_table(const orc_p3m_params* q, float H, float* table /*500*/, float* delta_sq);
/* Times `steps` run-loop iterations (drift, force, kick) of the port in float on nthreads host
 * threads; pair_stride S > 1 samples every S-th i-particle of the pair pass and scales its time.
 * out4 = {est. seconds per full step, PM s, cell-list s, sampled pair s} per step. */
int port_time_steps(const orc_pm_params* p, const orc_p3m_params* q, int n,
                    const float* state, const float* masses, int steps, int nthreads,
                    int pair_stride, double* out4);
/* port_time_steps with the y-sorted cell-list build sampled too: fill_stride F > 1 times the
 * reference's insertion sort on every F-th particle and scales it by F^2 (its cost is quadratic
 * in the cell populations); the pair pass then runs on the complete lists built by an
 * equivalent stable sort (untimed).  *wall (may be NULL) = seconds the call's steps took. */
int port_time_steps2(const orc_pm_params* p, const orc_p3m_params* q, int n,
                     const float* state, const float* masses, int steps, int nthreads,
                     int pair_stride, int fill_stride, double* out4, double* wall);

#ifdef __cplusplus
}
#endif
#endif
