// Compiled variants of the FP32 batched kernel: (solver, feature set,
// register-resident waves) for every layer count, the specialised ones at
// two resident-CTA bounds.  The host picks the smallest compiled feature
// set that covers a partition (CMTJ_FEAT_ALL with four waves covers
// everything), at the bound the caller asks for or else the default one.
#pragma once
#include "batch_f32.cuh"

#define CMTJ_BATCH_SPECIALISED(X, L)                                     \
  X(L, CMTJ_RK4, 0, 1)                                                   \
  X(L, CMTJ_RK4, CMTJ_FEAT_WAVES, 1)                                     \
  X(L, CMTJ_RK4, CMTJ_FEAT_WAVES | CMTJ_FEAT_OFFAXIS, 1)                 \
  X(L, CMTJ_EULER_HEUN, CMTJ_FEAT_WAVES, 1)                              \
  X(L, CMTJ_EULER_HEUN, CMTJ_FEAT_WAVES | CMTJ_FEAT_STT, 1)              \
  X(L, CMTJ_EULER_HEUN, CMTJ_FEAT_WAVES | CMTJ_FEAT_STT | CMTJ_FEAT_OFFAXIS, 1)
#define CMTJ_BATCH_GENERIC(X, L)                                         \
  X(L, CMTJ_RK4, CMTJ_FEAT_ALL, 4)                                       \
  X(L, CMTJ_EULER_HEUN, CMTJ_FEAT_ALL, 4)                                \
  X(L, CMTJ_HEUN, CMTJ_FEAT_ALL, 4)

// One entry per compiled kernel: solver, feature set, register-resident
// waves, its resident-CTA bound (min blocks per SM), whether it is the
// default instantiation of that (solver, features, waves) or the
// lower-occupancy one, and the kernel.
struct CmtjBatchVariant {
  int solver, feat, nw, mb, low;
  const void *fn;
};

#define CMTJ_VARIANT_ENTRY(L, S, F, N) \
  {S, F, N, cmtjf::min_blocks<L, S, F>(), 0, (const void *)&cmtjf::k_batch<L, S, F, N>},
#define CMTJ_VARIANT_ENTRY_LOW(L, S, F, N)          \
  {S, F, N, cmtjf::low_min_blocks<L, S, F>(), 1,    \
   (const void *)&cmtjf::k_batch<L, S, F, N, cmtjf::low_min_blocks<L, S, F>()>},
#define CMTJ_BATCH_VARIANT_TABLE(L)                                                       \
  {CMTJ_BATCH_SPECIALISED(CMTJ_VARIANT_ENTRY, L) CMTJ_BATCH_GENERIC(CMTJ_VARIANT_ENTRY, L) \
       CMTJ_BATCH_SPECIALISED(CMTJ_VARIANT_ENTRY_LOW, L)}

int cmtj_batch_variants_l1(const CmtjBatchVariant **out);
int cmtj_batch_variants_l2(const CmtjBatchVariant **out);
int cmtj_batch_variants_l3(const CmtjBatchVariant **out);
int cmtj_batch_variants_l4(const CmtjBatchVariant **out);
