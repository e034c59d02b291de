/*
 * cmtj_gpu.h -- C ABI of libcmtj_gpu.so, the GB300 macrospin solver.
 *
 * The reference (LemurPwned/cmtj) exposes its time loop through pybind11
 * class bindings (python/cmtj.cpp:35-513).  This library replaces the
 * compute behind those bindings with plain extern "C" entry points: every
 * argument is a plain pointer, a size or a POD struct defined below; device
 * buffers are owned by the caller (PyTorch tensors in the Python package)
 * and passed as raw device pointers together with a cudaStream_t (as void*).
 * No entry point throws; each returns CMTJ_OK or a negative error code and
 * leaves a message readable through cmtj_last_error().
 *
 * Units follow the reference: Ms in tesla, fields in A/m, lengths in metres,
 * times in seconds, current densities in A/m^2.
 */
#ifndef CMTJ_GPU_H_
#define CMTJ_GPU_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CMTJ_ABI_VERSION 2
#define CMTJ_MAX_LAYERS 8        /* FP64 plain form: layers per junction   */
#define CMTJ_MAX_LAYERS_F32 4    /* FP32 batched form: layers per junction */

/* Return codes. */
#define CMTJ_OK 0
#define CMTJ_ERR_ARG (-1)        /* bad argument (maps to ValueError)        */
#define CMTJ_ERR_CUDA (-2)       /* CUDA launch / runtime error              */
#define CMTJ_ERR_RUNTIME (-3)    /* reference runtime_error (RuntimeError)  */
#define CMTJ_ERR_LIMIT (-4)      /* size beyond a documented maximum         */

/* Per-junction status words written by the solvers. */
#define CMTJ_STATUS_OK 0u
#define CMTJ_STATUS_NAN 1u       /* "NAN magnetisation" (junction.hpp:1037) */
#define CMTJ_STATUS_NOT_RUN 2u   /* junction never reached (work queue bug)  */
#define CMTJ_STATUS_BAD_INPUT 3u /* layer count outside the supported range  */
/* Dormand-Prince, multi-layer: a layer rejected the step.  The reference
 * then takes the step size from Layer::hopt, which is never assigned (-1,
 * junction.hpp:259, 1700-1705); the forced acceptance that follows moves t
 * back by 1 s and the run does not terminate.  The GPU solver stops here. */
#define CMTJ_STATUS_DP_STALL 4u
#define CMTJ_STATUS_LIMIT 5u     /* Dormand-Prince: more than max_attempts steps */

/* ScalarDriver update types: drivers.hpp:18-29 (UpdateType). */
enum cmtj_update_type {
  CMTJ_DRV_CONSTANT = 0,
  CMTJ_DRV_PULSE = 1,
  CMTJ_DRV_SINE = 2,
  CMTJ_DRV_STEP = 3,
  CMTJ_DRV_POSINE = 4,
  CMTJ_DRV_HALFSINE = 5,
  CMTJ_DRV_TRAPEZOID = 6,
  CMTJ_DRV_GAUSSIMPULSE = 7,
  CMTJ_DRV_GAUSSSTEP = 8,
  /* custom (Python callback) drivers, drivers.hpp:294-303, are evaluated on
   * the host at every time the solver asks for and passed as a table of
   * [total_iterations][3] values at (t, t + dt/2, t + dt) of each step. */
  CMTJ_DRV_TABLE = 100
};

/* One ScalarDriver (drivers.hpp:63-305): the ten parameters of the
 * reference's ScalarDriver constructor, in its order. */
typedef struct cmtj_driver {
  int32_t update;          /* enum cmtj_update_type                        */
  int32_t reserved;
  int64_t table_offset;    /* CMTJ_DRV_TABLE: element offset in the table  */
  double constantValue, amplitude, frequency, phase, period, cycle;
  double timeStart, timeStop, edgeTime, steadyTime;
} cmtj_driver_t;           /* 96 bytes */

/* Driver slots of one Layer (junction.hpp:147-163).  Axial drivers take
 * three consecutive slots (x, y, z). */
enum cmtj_driver_slot {
  CMTJ_SLOT_TEMPERATURE = 0,
  CMTJ_SLOT_IEC_TOP = 1,
  CMTJ_SLOT_IEC_BOTTOM = 2,
  CMTJ_SLOT_IECQ_TOP = 3,
  CMTJ_SLOT_IECQ_BOTTOM = 4,
  CMTJ_SLOT_CURRENT = 5,
  CMTJ_SLOT_ANIS = 6,
  CMTJ_SLOT_ANIS2 = 7,
  CMTJ_SLOT_FL = 8,
  CMTJ_SLOT_DL = 9,
  CMTJ_SLOT_FL2 = 10,
  CMTJ_SLOT_DL2 = 11,
  CMTJ_SLOT_HEXT = 12,       /* 12, 13, 14 */
  CMTJ_SLOT_HOE = 15,        /* 15, 16, 17 */
  CMTJ_SLOT_HDMI = 18,       /* 18, 19, 20 */
  CMTJ_SLOT_HRES = 21,       /* 21, 22, 23 reserved interaction field */
  CMTJ_SLOT_IDMI_TOP = 24,   /* 24, 25, 26 */
  CMTJ_SLOT_IDMI_BOTTOM = 27,/* 27, 28, 29 */
  CMTJ_NUM_SLOTS = 30
};

/* Reference enum (junction.hpp:141). */
enum cmtj_reference { CMTJ_REF_NONE = 0, CMTJ_REF_FIXED = 1, CMTJ_REF_TOP = 2, CMTJ_REF_BOTTOM = 3 };
/* SolverMode (junction.hpp:143). */
enum cmtj_solver { CMTJ_EULER_HEUN = 0, CMTJ_RK4 = 1, CMTJ_DORMAND_PRINCE = 2, CMTJ_HEUN = 3 };
/* Junction MRmode (junction.hpp:1144). */
enum cmtj_mr_mode { CMTJ_MR_NONE = 0, CMTJ_MR_CLASSIC = 1, CMTJ_MR_STRIP = 2,
                   /* FP32 form only: Rx = sum_l Rx0 + AMR_X mx^2 + SMR_X my^2, the
                    * series formula of cmtj/utils/resistance.py:121-150 */
                   CMTJ_MR_SERIES = 3 };

/* AdaptiveIntegrationParams<double> (junction.hpp:125-139) of one layer.
 * prev_error_ratio and integral_error are the PID controller's state, which
 * the solver updates in place like mag. */
typedef struct cmtj_adaptive {
  double abs_tol, rel_tol, max_factor, min_factor, safety_factor;
  double ki, kp, kd;
  double prev_error_ratio, integral_error;
  int32_t use_pid_control, reserved;
} cmtj_adaptive_t;         /* 88 bytes */

/* One Layer<double> (junction.hpp:145-258), as the solver needs it. */
typedef struct cmtj_layer {
  double mag[3];             /* current magnetisation (the solver state)   */
  double anis[3];
  double ref[3];             /* referenceLayer                             */
  double ref2[3];            /* secondaryReferenceLayer                    */
  double demag[9];           /* row-major 3x3                              */
  double dipole_top[9];
  double dipole_bottom[9];
  double Ms, thickness, cellSurface, cellVolume, damping;
  double fieldLikeTorque, dampingLikeTorque;   /* static SOT (createSOTLayer) */
  double slonczewski, beta, kappa, spinPolarisation; /* STT                */
  int32_t referenceType;     /* enum cmtj_reference                        */
  int32_t includeSTT, includeSOT, dynamicSOT, alternativeSTT, temperatureSet;
  uint32_t seed_lo, seed_hi; /* Philox4x32-10 key of this layer's noise    */
  uint64_t noise_step;       /* Philox step counter at iteration 0         */
  cmtj_driver_t drv[CMTJ_NUM_SLOTS];
  cmtj_adaptive_t adaptive;  /* Dormand-Prince step control               */
  /* Derived by the host from the fields above, with the reference's own
   * expressions evaluated once (the solver would recompute the same bits at
   * every call): 1/(1+damping^2) (solveLLG, junction.hpp:719),
   * -gyro/(1+damping^2) (stochasticTorque, 826), Ms/mu0 (the demag and
   * dipole scale, 54-72), and which field terms are identically zero
   * (CMTJ_ZERO_*): adding an exact zero changes no value, so the solver
   * skips them. */
  double conv_term, stoch_conv, ms_over_mu0;
  uint32_t zero_terms, reserved2;
  /* Buffered 1/f^alpha noise of this run (setAlphaNoise, getOneFVector,
   * junction.hpp:406-424, 1130-1136): null for none, else the samples of
   * iterations 0 .. alpha_len-1 in three rows (x, y, z) of alpha_len floats
   * each, as cmtj_alpha_noise_f32 writes them.  alpha_axis is the Axis:
   * 0, 1, 2 use that component alone; 3 (all) uses the normalised sample
   * vector (VectorAlphaNoise::tickVector, noise.hpp:280-290).  The
   * Euler-Heun and Heun runners add alpha_scale times it to the layer's
   * thermal dW at iteration i (junction.hpp:1727, 1793). */
  const float *alpha_buf;
  double alpha_scale;
  uint32_t alpha_len;
  int32_t alpha_axis;
} cmtj_layer_t;

#define CMTJ_ZERO_DIPOLE 1u  /* both dipole tensors are zero                 */
#define CMTJ_ZERO_IDMI 2u    /* the six IDMI driver slots are constant 0     */
#define CMTJ_ZERO_K2 4u      /* second-order anisotropy is constant 0        */
#define CMTJ_ZERO_J2 8u      /* both quadratic IEC drivers are constant 0    */

/* One Junction<double> (junction.hpp:1139-1243). */
typedef struct cmtj_junction {
  int32_t n_layers;
  int32_t mr_mode;           /* enum cmtj_mr_mode                          */
  int32_t layer_offset;      /* index of its first layer in the layer array */
  int32_t reserved;
  double Rp, Rap;
  double Rx0[CMTJ_MAX_LAYERS], Ry0[CMTJ_MAX_LAYERS];
  double AMR_X[CMTJ_MAX_LAYERS], AMR_Y[CMTJ_MAX_LAYERS];
  double SMR_X[CMTJ_MAX_LAYERS], SMR_Y[CMTJ_MAX_LAYERS];
  double AHE[CMTJ_MAX_LAYERS];
} cmtj_junction_t;

/* PhysicalConstants (constants.hpp:6-55), passed per launch because the
 * reference lets Python change them at run time. */
typedef struct cmtj_constants {
  double mu0, gyro, TtoAm, hbar, echarge, kB;
} cmtj_constants_t;

/* Arguments of Junction::runSimulation (junction.hpp:1948-1981) after the
 * host has resolved them exactly as the reference does:
 *   total_iterations = (unsigned)(totalTime / timeStep)
 *   write_every      = (unsigned)(writeFrequency / timeStep)
 *   solver           = getSolver(...) result (junction.hpp:1891-1931).
 * Dormand-Prince (junction.hpp:1982-2045) reads total_time, write_frequency
 * and time_step (the first step) instead of the two counts; its log holds at
 * most floor(total_time / write_frequency) + 2 rows. */
typedef struct cmtj_sim_params {
  double time_step;
  uint32_t total_iterations;
  uint32_t write_every;
  uint32_t n_log;            /* fixed step: ceil(total_iterations/write_every);
                                Dormand-Prince: log capacity in rows         */
  int32_t solver;            /* enum cmtj_solver                             */
  int32_t calculate_energies;
  int32_t log_width;         /* doubles per log row, cmtj_log_width()       */
  cmtj_constants_t c;
  double total_time, write_frequency;
  uint64_t max_attempts;     /* Dormand-Prince: step attempts before CMTJ_STATUS_LIMIT */
  int32_t max_layers;        /* fixed step: an upper bound on n_layers over the
                                batch (0: CMTJ_MAX_LAYERS); a junction with more
                                layers gets CMTJ_STATUS_BAD_INPUT            */
  int32_t lanes_per_layer;   /* fixed step: 1 (a layer per lane) or 4 (a layer's
                                x, y, z on three lanes); 0: the library picks 4
                                for batches up to two quad warps per SM
                                sub-partition, else 1.  Results are the same. */
  int32_t arithmetic;        /* enum cmtj_arithmetic                         */
  int32_t reserved;          /* 0                                            */
} cmtj_sim_params_t;

/* How cmtj_run_simulation_f64 evaluates fixed-step RK4 layers.
 *   CMTJ_ARITH_REFERENCE  the reference's operations in its order, no FMA
 *                         contraction: the reference's bits (the default).
 *   CMTJ_ARITH_FUSED      a warp whose layers are all field-only (no dipole,
 *                         IDMI, K2, biquadratic IEC, STT or SOT) with constant
 *                         anisotropy and IEC drivers, and without
 *                         calculate_energies, forms the field as
 *                         H = Hconst + A m (A = (2K/Ms) k k^T - N Ms/mu0, one
 *                         constant matrix per layer), contracts products into
 *                         FMAs and normalises |m| by a series in |m|^2 - 1.
 *                         Each result differs from the reference's in the last
 *                         bits; the difference a run accumulates depends on
 *                         how sensitive its trajectory is (the library's tests
 *                         state the bound they check).  Other warps, other
 *                         solvers, stacks and groups use the reference
 *                         arithmetic. */
enum cmtj_arithmetic { CMTJ_ARITH_REFERENCE = 0, CMTJ_ARITH_FUSED = 1 };

/* Log row layout (per junction, per row): for each layer l, either 3
 * doubles (mx, my, mz) or, with calculate_energies, CMTJ_ENERGY_COLS doubles
 * in the order of junction.hpp:1589-1616:
 *   K, K2, Jbottom, Jtop, I, Hext[3], Hiec[3], Hanis[3], Hdemag[3], Hth[3],
 *   Hfl[3], Hdl[3], mx, my, mz
 * followed by 3 magnetoresistance doubles (R | R_a_b | Rx, Ry, Rz) and the
 * time.  Log buffer: [n_junctions][n_log][log_width] doubles. */
#define CMTJ_ENERGY_COLS 29
int cmtj_log_width(int n_layers, int calculate_energies);

/* ---------------------------------------------------------------------- */
/* Library.                                                               */
/* ---------------------------------------------------------------------- */
int cmtj_abi_version(void);
/* Message of the last failing call on this host thread ("" if none). */
const char *cmtj_last_error(void);
/* Device properties the host planner needs: SM count and compute capability. */
int cmtj_device_info(int device, int32_t *sm_count, int32_t *cc_major, int32_t *cc_minor);
/* sizeof of the structs of this header, in this order: cmtj_driver_t,
 * cmtj_layer_t, cmtj_junction_t, cmtj_constants_t, cmtj_sim_params_t,
 * cmtj_wave_t, cmtj_f32_layer_t, cmtj_f32_junction_t, cmtj_f32_state_t,
 * cmtj_f32_params_t, cmtj_stack_t, cmtj_group_t, cmtj_pair_t (the first
 * n <= 13); lets a binding check
 * its mirror of the layout. */
int cmtj_struct_sizes(int32_t *sizes, int32_t n);

/* ---------------------------------------------------------------------- */
/* FP64 plain form.                                                        */
/* ---------------------------------------------------------------------- */
/* Junction::runSimulation (core/junction.hpp:1948-2056) for n_junctions
 * independent junctions, FP64, arithmetic in the reference's order with no
 * FMA contraction.  Fixed step: each junction's layers side by side on
 * lanes (p->max_layers, p->lanes_per_layer choose the layout, not the
 * result); Dormand-Prince: one device thread per junction.
 *   d_junctions  [n_junctions] cmtj_junction_t           (device, read)
 *   d_layers     [total layers] cmtj_layer_t; .mag is updated in place
 *   d_tables     custom-driver tables (device, may be NULL)
 *   d_log        [n_junctions][p->n_log][p->log_width] doubles (device, write)
 *   d_status     [n_junctions][2] uint32: {status word, log rows written}
 *   stream       cudaStream_t (NULL = legacy default stream)               */
int cmtj_run_simulation_f64(const cmtj_junction_t *d_junctions, int32_t n_junctions,
                            cmtj_layer_t *d_layers, const double *d_tables,
                            const cmtj_sim_params_t *p, double *d_log,
                            uint32_t *d_status, void *stream);

/* ---------------------------------------------------------------------- */
/* Electrically coupled stacks (core/stack.hpp), FP64 plain form.          */
/* ---------------------------------------------------------------------- */
enum cmtj_stack_kind { CMTJ_STACK_SERIES = 0, CMTJ_STACK_PARALLEL = 1 };

/* One SeriesStack / ParallelStack (stack.hpp:16-480). */
typedef struct cmtj_stack {
  int32_t first_junction;    /* its junctions: [first, first + n_junctions) */
  int32_t n_junctions;       /* 2 .. 256                                     */
  int32_t kind;              /* enum cmtj_stack_kind                          */
  int32_t use_kcl;           /* runSimulationKCL (1) or NonKCL (0)            */
  int32_t delayed;           /* non-KCL: coupling from frozen magnetisations  */
  int32_t single_layer_runner; /* last junction has one layer (RK4): every
                                  junction steps only its layer 0 (stack.hpp:48-57) */
  int32_t coupling_offset, n_coupling; /* 1 value, or n_junctions-1 values  */
  double phase_offset;
  double pol[3];             /* polarisation when not a 2-layer stack        */
  cmtj_driver_t current;     /* the coupled current driver                    */
} cmtj_stack_t;

/* Stack::runSimulation (stack.hpp:311-423) for n_stacks stacks, one CTA
 * each; each junction's layers on lanes when the widest stack fits a
 * 256-thread CTA that way, else one thread per junction (same results).
 * d_top_bottom[2*j] / [2*j+1]: index (within junction j) of the
 * topId layer and of the bottomId layer (-1: use cmtj_stack_t.pol).
 * Junction logs as cmtj_run_simulation_f64; the stack log is
 * [n_stacks][p->n_log][stack_width] doubles per row: Resistance,
 * I_0..I_{N-1}, C_0_1..C_{N-2}_{N-1}, time (stack_width >= 2*max_junctions+1). */
int cmtj_run_stack_f64(const cmtj_stack_t *d_stacks, int32_t n_stacks, const double *d_couplings,
                       const cmtj_junction_t *d_junctions, const int32_t *d_top_bottom, cmtj_layer_t *d_layers,
                       const double *d_tables, const cmtj_sim_params_t *p, double *d_log, double *d_stack_log,
                       int32_t stack_width, int32_t max_junctions, uint32_t *d_status, void *stream);

/* ---------------------------------------------------------------------- */
/* Dipole-coupled groups: GroupInteraction (reservoir.hpp:122-245).        */
/* ---------------------------------------------------------------------- */
/* The interaction function of a group (reservoir.hpp:61-122). */
enum cmtj_interaction {
  CMTJ_INTERACTION_NULL = 0,    /* nullDipoleInteraction                    */
  CMTJ_INTERACTION_DIPOLE = 1,  /* computeDipoleInteraction (the default)   */
  CMTJ_INTERACTION_NOUMRA = 2   /* computeDipoleInteractionNoumra           */
};

typedef struct cmtj_group {
  int32_t first_junction;       /* its junctions: [first, first + n_junctions) */
  int32_t n_junctions;          /* 1 .. 256                                     */
  int32_t interaction;          /* enum cmtj_interaction                        */
  int32_t single_layer_runner;  /* RK4 with runSingleLayerSolver for every
                                   junction (the last one has one layer)      */
  int64_t pair_offset;          /* its n*n cmtj_pair_t records, row i = target */
} cmtj_group_t;                 /* 24 bytes */

/* The fixed geometry of the ordered pair (i, j) of a group (the field on i
 * from j), formed once on the host with the reference's own expressions:
 *   DIPOLE: g = (rij.x, rij.y, rij.z, |rij|^3, |rij|^5) with rij = r_i - r_j
 *           (computeDipoleInteraction, reservoir.hpp:77-97); scale =
 *           (Ms_j / mu0) * thickness_j * cellSurface_j
 *   NOUMRA: g = the 3x3 tensor of getDipoleTensorFromRelPositions (37-57),
 *           row-major; scale = Ms_j * V_j / mu0 (calculate_tensor_interaction)
 * so the device evaluates only the part that depends on m_j. */
typedef struct cmtj_pair {
  double g[9];
  double scale;
} cmtj_pair_t;                  /* 80 bytes */

/* GroupInteraction::runSimulation for n_groups groups, one CTA each; each
 * junction's layers on lanes when the widest group fits a 256-thread CTA
 * that way, else one thread per junction (same results).  Every step: each
 * junction's field from all others'
 * top-layer magnetisations (frozen at step start) is summed in index order
 * and set as its top layer's reserved interaction field (the HRES driver
 * slots, setLayerReservedInteractionField), then every junction steps.
 * d_top[j]: index (within junction j) of the topId layer.  Logs and status
 * as cmtj_run_simulation_f64 (calculateEnergies off). */
int cmtj_run_group_f64(const cmtj_group_t *d_groups, int32_t n_groups, const cmtj_pair_t *d_pairs,
                       const cmtj_junction_t *d_junctions, const int32_t *d_top, cmtj_layer_t *d_layers,
                       const double *d_tables, const cmtj_sim_params_t *p, double *d_log, int32_t max_junctions,
                       uint32_t *d_status, void *stream);

/* ---------------------------------------------------------------------- */
/* FP32 batched form.                                                      */
/* ---------------------------------------------------------------------- */
/* Many independent junctions (1-4 layers each, uneven durations and driver
 * sets) in one persistent launch.  The host lowers each junction into the
 * records below: constant drivers are folded into per-layer coefficients
 * (already divided by Ms, Ms*t, mu0 as the field terms need), and each
 * time-dependent driver becomes one cmtj_wave_t.  m, fields and torques are
 * FP32 with |m| renormalised every step; driver time enters through integer
 * step counts and 64-bit fixed-point phases, so no FP32 time variable ever
 * accumulates rounding. */

/* Wave kinds: the time-dependent part of a ScalarDriver (drivers.hpp:262-305). */
enum cmtj_wave_kind {
  CMTJ_WAVE_SINE = 2, CMTJ_WAVE_STEP = 3, CMTJ_WAVE_POSINE = 4, CMTJ_WAVE_HALFSINE = 5,
  CMTJ_WAVE_PULSE = 1, CMTJ_WAVE_TRAPEZOID = 6, CMTJ_WAVE_GAUSSIMPULSE = 7, CMTJ_WAVE_GAUSSSTEP = 8
};
/* Wave targets: which term of the field/torque the wave adds to. */
enum cmtj_wave_target {
  CMTJ_TGT_HX = 0, CMTJ_TGT_HY = 1, CMTJ_TGT_HZ = 2,   /* Hext+Hoe+Hdmi+Hres sum (A/m)      */
  CMTJ_TGT_K = 3,                                       /* 2K/Ms                             */
  CMTJ_TGT_K2 = 4,                                      /* 4K2/Ms                            */
  CMTJ_TGT_JB = 5, CMTJ_TGT_JT = 6,                     /* J/(Ms t) bottom / top             */
  CMTJ_TGT_J2B = 7, CMTJ_TGT_J2T = 8,                   /* 2 J2/(Ms t) bottom / top          */
  CMTJ_TGT_I = 9,                                       /* current density (STT, static SOT) */
  CMTJ_TGT_FL = 10, CMTJ_TGT_DL = 11, CMTJ_TGT_FL2 = 12, CMTJ_TGT_DL2 = 13, /* dynamic SOT   */
  CMTJ_TGT_T = 14,                                      /* temperature (K)                   */
  CMTJ_NUM_TGT = 15
};

/* One time-dependent driver.  Time is t_s = i*dt + s*dt/2 for step i and
 * RK stage s in {0, 1, 2}.
 *   SINE/POSINE/HALFSINE: phase (cycles, Q0.64) = ph0 + i*dph + s*dph_half;
 *                         value = amp * sin(2 pi phase)
 *   PULSE:                phase (Q0.64 of t/period) as above; on while
 *                         phase <= cycle (thr32 compares the top 32 bits)
 *   STEP:                 on while i in [on[s], off[s]] (inclusive; the host
 *                         found these by evaluating the reference's FP64
 *                         comparisons)
 *   TRAPEZOID/GAUSS*:     tau = t - t0 = (i - i0)*dt + s*dt/2 + r0           */
typedef struct cmtj_wave {
  int32_t target, kind;
  float amp;              /* amplitude, scaled like the target term            */
  float p0, p1, p2;       /* TRAPEZOID: edge, steady, r0; GAUSSIMPULSE: 1/sigma, -, r0;
                              GAUSSSTEP: 1/(sqrt2 sigma), -, r0                  */
  uint32_t thr32;         /* PULSE duty threshold (Q0.32)                      */
  int32_t i0;             /* TRAPEZOID/GAUSS*: step index nearest t0            */
  uint64_t ph0, dph, dph_half;  /* SINE family / PULSE (Q0.64 cycles)           */
  uint32_t on[3], off[3]; /* STEP: inclusive step-index window per stage        */
  int32_t layer_mask;     /* bit l: the wave drives layer l                     */
  int32_t reserved;
} cmtj_wave_t;            /* 88 bytes */

#define CMTJ_MAX_WAVES 4  /* distinct time-dependent drivers per junction     */

/* Layer record of the FP32 form.  Field terms (junction.hpp:580-701) become:
 *   Hanis = anis * (kc * (anis.m)),  Hanis2 = anis * (k2c * (anis.m)^3)
 *   Hdemag = demag . m,  Hdipole = dip_b . m_bottom + dip_t . m_top
 *   Hiec = m_b * (jb + j2b (m_b.m)) + m_t * (jt + j2t (m_t.m))
 *   Hidmi = m_b x dmi_b + m_t x dmi_t          (= -(D x m_c)/(Ms t))
 *   H = h0 + waves + Hanis + Hanis2 + Hiec + Hidmi - Hdemag - Hdipole
 * and the torque (716-815): dm/dt = gam (m x H + alpha m x (m x H)) + STT/SOT. */
typedef struct cmtj_f32_layer {
  float m[3];             /* initial m, as stored (not renormalised)           */
  float anis[3];
  float kc, k2c;          /* 2K/Ms, 4K2/Ms (constant parts)                    */
  float demag[9];         /* N * Ms/mu0                                        */
  float dip_b[9], dip_t[9];
  float h0[3];            /* constant part of Hext + Hoe + Hdmi + Hres         */
  float jb, jt, j2b, j2t; /* J/(Ms t), 2 J2/(Ms t) constant parts              */
  float dmi_b[3], dmi_t[3];
  float gam, alpha;       /* -gamma/(1+alpha^2), alpha                         */
  float ref[3], ref2[3];
  int32_t ref_type;       /* enum cmtj_reference                               */
  int32_t flags;          /* CMTJ_F32_STT | _SOT | _SOT_STATIC | _ALT_STT      */
  float stt_c;            /* gamma*hbar/(e Ms t (1+alpha^2))                   */
  float stt_p, stt_l, stt_beta, stt_kappa; /* P, lambda, beta, kappa           */
  float i0;               /* constant current density                          */
  float fl0, dl0, fl20, dl20; /* SOT: dynamic constants, or static torques/A   */
  float sig_c;            /* 2 alpha kB / (Ms V gamma): sigma = sqrt(sig_c*T)  */
  float t0;               /* constant temperature                              */
  uint32_t seed_lo, seed_hi;
  uint32_t noise_step_lo, noise_step_hi;
  /* time-step prefactors, each formed in FP64 and rounded once:
   *   gdt  = gam * dt,      stt_cdt  = stt_c * dt        (Euler-Heun, Heun)
   *   gdt6 = gam * dt / 6,  stt_cdt6 = stt_c * dt / 6    (RK4: with k' = k/6
   *   every RK4 constant is an exact small integer: m + 3k', m + 6k',
   *   m + k1' + 2k2' + 2k3' + k4', so no weight or dt rounding drifts
   *   the precession phase over long runs) */
  float gdt, gdt6, stt_cdt, stt_cdt6;
} cmtj_f32_layer_t;

#define CMTJ_F32_STT 1
#define CMTJ_F32_SOT 2
#define CMTJ_F32_SOT_STATIC 4
#define CMTJ_F32_ALT_STT 8

/* Junction header of the FP32 form. */
typedef struct cmtj_f32_junction {
  int32_t n_layers, mr_mode;
  int32_t layer_offset;   /* first layer in the cmtj_f32_layer_t array         */
  uint32_t n_steps;       /* iterations of this junction                      */
  uint32_t win_start;     /* first step included in the on-device reductions */
  uint32_t log_offset;    /* start of this junction's log row, in 16-byte
                             granules (units of 4 floats) of the log buffer  */
  float Rp, Rap;
  float Rx0[CMTJ_MAX_LAYERS_F32], Ry0[CMTJ_MAX_LAYERS_F32];
  float AMR_X[CMTJ_MAX_LAYERS_F32], AMR_Y[CMTJ_MAX_LAYERS_F32];
  float SMR_X[CMTJ_MAX_LAYERS_F32], SMR_Y[CMTJ_MAX_LAYERS_F32];
  float AHE[CMTJ_MAX_LAYERS_F32];
  float mix_w[CMTJ_MAX_LAYERS_F32]; /* weights of the mixed log channel        */
  uint64_t vsd_ph0, vsd_dph;        /* I(t) = sin(2 pi (vsd_ph0 + i vsd_dph))  */
  int32_t n_waves;
  uint32_t red_total;     /* reduction samples the whole run takes: sample k
                             of the weighted sum gets red_weights[red_total-1-k] */
  cmtj_wave_t waves[CMTJ_MAX_WAVES];
} cmtj_f32_junction_t;

/* Per-junction resumable state and on-device reductions (FP32 form). */
typedef struct cmtj_f32_state {
  float m[CMTJ_MAX_LAYERS_F32][3];
  uint32_t step;          /* next iteration to run                             */
  uint32_t status;        /* CMTJ_STATUS_*                                     */
  uint32_t n_logged;      /* log samples written so far                        */
  uint32_t n_red;         /* samples in the reductions                         */
  float r_sum, r_c;       /* compensated (Neumaier) sum of R                   */
  float v_sum, v_c;       /* compensated sum of I(t) * R(t)                    */
  float vw_sum, vw_c;     /* compensated sum of w_k I R (params.red_weights)   */
} cmtj_f32_state_t;

/* What the kernel logs every log_every steps (from step 0, like the
 * reference's i % writeEvery == 0). */
enum cmtj_log_mode {
  CMTJ_LOG_NONE = 0,
  CMTJ_LOG_M = 1,         /* all components of every layer: 3*n_layers floats  */
  CMTJ_LOG_MIX = 2,       /* sum_l mix_w[l] * m_l[log_axis]: 1 float           */
  CMTJ_LOG_R = 3          /* R (classic) or Rx (strip): 1 float                */
};

typedef struct cmtj_f32_params {
  double dt;              /* time step (s)                                     */
  uint32_t chunk_steps;   /* max iterations per junction in this launch
                           * (0xffffffff: run to the end).  With a log, a
                           * multiple of log_every * log_tile, so that every
                           * chunk ends on a whole log tile (else
                           * CMTJ_ERR_ARG)                                    */
  int32_t solver;         /* CMTJ_RK4, CMTJ_EULER_HEUN or CMTJ_HEUN            */
  int32_t log_mode, log_axis;
  uint32_t log_every;     /* 0: no log                                         */
  uint32_t log_tile;      /* samples staged per thread before a bulk store     */
  uint32_t red_every;     /* reduction cadence in steps (0: none)              */
  int32_t reserved;
  /* Optional (null: off) weights of a second I(t) R(t) sum.  With w the step
   * response of a causal linear filter started at rest, sum_k w[N-1-k] x_k
   * / N is the mean of the filtered x: the Butterworth low-pass mean of
   * cmtj/utils/resistance.py:12-22 (compute_sd) without a per-step filter. */
  const float *red_weights;
} cmtj_f32_params_t;

/* Kernel variant of a batch partition: n_layers (1-4), solver, and the
 * CMTJ_FEAT_* terms its junctions use (bits 0-15 of `features`; bits 16-23:
 * waves per junction; bits 24-27: the resident-CTA bound asked for, 0 for
 * the variant's default).  A variant that was not compiled falls back to
 * the generic one of the same layer count and solver.  The specialised
 * variants are compiled at two bounds: their default and a lower one (more
 * registers per thread), for batches too small to fill the GPU. */
#define CMTJ_FEAT_FULL_DEMAG 1
#define CMTJ_FEAT_DIPOLE 2
#define CMTJ_FEAT_IDMI 4
#define CMTJ_FEAT_K2 8
#define CMTJ_FEAT_STT 16
#define CMTJ_FEAT_SOT 32
#define CMTJ_FEAT_WAVES 64         /* waves on the field (HX, HY, HZ) and, with
                                      STT or SOT, on I / FL / DL / FL2 / DL2      */
#define CMTJ_FEAT_SCALAR_WAVES 128 /* waves on K, K2, J*, T                      */
#define CMTJ_FEAT_IEC2 256         /* quadratic (biquadratic) IEC, J2 != 0        */
#define CMTJ_FEAT_OFFAXIS 512      /* an anisotropy axis with more than one
                                    * non-zero component.  Without it, K2, full
                                    * demag and scalar waves, anisotropy and
                                    * demag fold into one diagonal tensor.     */
#define CMTJ_FEAT_ALL 1023

/* Runs every junction of one partition (all with n_layers layers and the
 * same solver) for up to p->chunk_steps iterations, resuming from d_state
 * (state.step == 0 starts from the record).  Junctions are taken from
 * d_order[0..n) through a work-stealing ticket in d_ticket (one uint32,
 * zeroed by this call on `stream`).
 *   d_log  one row of ceil4(samples) * channels floats per junction,
 *          starting at float 4 * log_offset (16-byte aligned).
 *   grid_blocks <= 0 picks one persistent wave of the device.              */
int cmtj_batch_run_f32(const cmtj_f32_junction_t *d_junctions, const cmtj_f32_layer_t *d_layers,
                       cmtj_f32_state_t *d_state, const int32_t *d_order, int32_t n, int32_t n_layers,
                       int32_t features, const cmtj_f32_params_t *p, float *d_log, uint32_t *d_ticket,
                       int32_t grid_blocks, void *stream);

/* Feature set actually compiled for (n_layers, solver, features): the
 * variant cmtj_batch_run_f32 will run, as features | waves << 16 |
 * resident-CTA bound << 24. */
int cmtj_batch_variant_f32(int32_t n_layers, int32_t solver, int32_t features);

/* No counterpart in the reference (launch tuning): the resident-CTA bounds
 * compiled for the variant of (n_layers, solver, features), default first,
 * into bounds[0..n); returns how many, or CMTJ_ERR_ARG. */
int cmtj_batch_bounds_f32(int32_t n_layers, int32_t solver, int32_t features, int32_t *bounds, int32_t n);

/* No counterpart in the reference: an allocation-free form of
 * cmtj_batch_run_f32 for callers that cannot call cudaMalloc (code running
 * under CUDA graph capture, real-time threads that must not take the
 * driver's allocation locks, hosts that give a plugin a fixed memory arena).
 * Same arguments and results, except that the work-stealing ticket lives in
 * a static device array inside the library, CMTJ_NOALLOC_TICKET_SLOTS
 * tickets (256 bytes per GPU, held until the process exits), chosen by
 * ticket_slot; a slot outside [0, CMTJ_NOALLOC_TICKET_SLOTS) returns
 * CMTJ_ERR_LIMIT.  The caller still passes every input and output buffer.
 * The first call on a device resolves the array's device address
 * (cudaGetSymbolAddress) with that device current, so make it before any
 * stream capture.  The address is cached per device together with the id of
 * the context it was resolved in, and resolved again when that context
 * changes (after cudaDeviceReset): the first call after such a reset is a
 * set-up call too.  Each call zeroes its slot on `stream` before launching;
 * calls that overlap on the GPU and use the same slot race on its ticket. */
#define CMTJ_NOALLOC_TICKET_SLOTS 64
int cmtj_batch_run_f32_noalloc(const cmtj_f32_junction_t *d_junctions, const cmtj_f32_layer_t *d_layers,
                               cmtj_f32_state_t *d_state, const int32_t *d_order, int32_t n, int32_t n_layers,
                               int32_t features, const cmtj_f32_params_t *p, float *d_log, int32_t ticket_slot,
                               int32_t grid_blocks, void *stream);

/* ---------------------------------------------------------------------- */
/* Buffered 1/f^alpha noise (core/noise.hpp:138-241).                      */
/* ---------------------------------------------------------------------- */
/* One buffer row of BufferedAlphaNoise::fillBuffer: n white draws of
 * standard deviation `std` coloured by the 1/f^alpha filter.  The white
 * draw m is normal `component` (0, 1 or 2) of the Philox4x32-10 block with
 * key (seed_lo, seed_hi) and counter {counter + m, 0xA1F4, 0}, the thermal
 * stream's Box-Muller transform on an independent counter tag. */
typedef struct cmtj_alpha_noise {
  double alpha;           /* exponent in [0, 2] (outside: NaN samples)      */
  double std;             /* standard deviation of the white draws          */
  uint32_t seed_lo, seed_hi;
  uint64_t counter;
  int32_t component;
  int32_t reserved;
} cmtj_alpha_noise_t;     /* 40 bytes */

#define CMTJ_ALPHA_MAX_LEN 8388608u  /* samples per buffer (2^23)          */

/* Scratch bytes per buffer row for buffers of n samples (0 when n is 0 or
 * above CMTJ_ALPHA_MAX_LEN): three complex float rows of the power-of-two
 * FFT size M >= 2n - 1 and 64 bytes. */
size_t cmtj_alpha_noise_scratch_bytes(uint32_t n);

/* BufferedAlphaNoise::fillBuffer (noise.hpp:186-225) for n_buffers rows:
 * d_out[r*n .. r*n+n) = the reference's buffer of d_specs[r] (a device
 * array).  d_white, when not null, holds the white draws [n_buffers][n]
 * instead of the Philox ones.  The caller's 16-byte aligned d_scratch of
 * scratch_bytes holds k >= 1 rows' scratch; rows are processed k at a time.
 * Samples follow the reference's algorithm exactly (weights by its float
 * recurrence, the halved bins 0 and n-1 and the dropped upper half),
 * computed as one FFT convolution plus the two top bins in FP64. */
int cmtj_alpha_noise_f32(const cmtj_alpha_noise_t *d_specs, int32_t n_buffers, uint32_t n, const float *d_white,
                         float *d_out, void *d_scratch, size_t scratch_bytes, void *stream);

/* ---------------------------------------------------------------------- */
/* On-device reductions.                                                   */
/* ---------------------------------------------------------------------- */
/* compute_spectrum_strip (cmtj/utils/procedures.py:28-39): for each of
 * n_rows log rows (row r starts at d_series + r*row_stride and holds
 * series_len samples), |FFT| of its last n_fft samples (n_fft a power of two,
 * <= 8192), bins [bin_lo, bin_hi) written to d_out[r*(bin_hi-bin_lo) ...]. */
int cmtj_spectrum_f32(const float *d_series, int64_t row_stride, int32_t n_rows, int32_t series_len,
                      int32_t n_fft, int32_t bin_lo, int32_t bin_hi, float *d_out, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* CMTJ_GPU_H_ */
