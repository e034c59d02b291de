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

#define CMTJ_ABI_VERSION 1
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
enum cmtj_mr_mode { CMTJ_MR_NONE = 0, CMTJ_MR_CLASSIC = 1, CMTJ_MR_STRIP = 2 };

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
} cmtj_layer_t;

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
 *   solver           = getSolver(...) result (junction.hpp:1891-1931). */
typedef struct cmtj_sim_params {
  double time_step;
  uint32_t total_iterations;
  uint32_t write_every;
  uint32_t n_log;            /* rows written: ceil(total_iterations/write_every) */
  int32_t solver;            /* enum cmtj_solver (RK4, EULER_HEUN, HEUN)   */
  int32_t calculate_energies;
  int32_t log_width;         /* doubles per log row, cmtj_log_width()       */
  cmtj_constants_t c;
} cmtj_sim_params_t;

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
/* sizeof of the structs above, in this order: cmtj_driver_t, cmtj_layer_t,
 * cmtj_junction_t, cmtj_constants_t, cmtj_sim_params_t (n <= 5 entries);
 * lets a binding check its mirror of the layout. */
int cmtj_struct_sizes(int32_t *sizes, int32_t n);

/* ---------------------------------------------------------------------- */
/* FP64 plain form.                                                        */
/* ---------------------------------------------------------------------- */
/* Junction::runSimulation (core/junction.hpp:1948-2056) for n_junctions
 * independent junctions, FP64, one device thread per junction, arithmetic
 * in the reference's order with no FMA contraction.
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

#ifdef __cplusplus
}
#endif
#endif /* CMTJ_GPU_H_ */
