// Compiled variants of the FP32 batched kernel: (solver, feature set,
// register-resident waves) for every layer count.  The host picks the
// smallest compiled feature set that covers a partition; CMTJ_FEAT_ALL with
// four waves covers everything.
#pragma once
#include "batch_f32.cuh"

#define CMTJ_BATCH_VARIANTS(X, L)                                        \
  X(L, CMTJ_RK4, 0, 1)                                                   \
  X(L, CMTJ_RK4, CMTJ_FEAT_WAVES, 1)                                     \
  X(L, CMTJ_RK4, CMTJ_FEAT_WAVES | CMTJ_FEAT_OFFAXIS, 1)                 \
  X(L, CMTJ_RK4, CMTJ_FEAT_ALL, 4)                                       \
  X(L, CMTJ_EULER_HEUN, CMTJ_FEAT_WAVES, 1)                              \
  X(L, CMTJ_EULER_HEUN, CMTJ_FEAT_WAVES | CMTJ_FEAT_STT, 1)              \
  X(L, CMTJ_EULER_HEUN, CMTJ_FEAT_WAVES | CMTJ_FEAT_STT | CMTJ_FEAT_OFFAXIS, 1) \
  X(L, CMTJ_EULER_HEUN, CMTJ_FEAT_ALL, 4)                                \
  X(L, CMTJ_HEUN, CMTJ_FEAT_ALL, 4)

struct CmtjBatchVariant {
  int solver, feat, nw;
  const void *fn;
};

#define CMTJ_VARIANT_ENTRY(L, S, F, N) {S, F, N, (const void *)&cmtjf::k_batch<L, S, F, N>},

int cmtj_batch_variants_l1(const CmtjBatchVariant **out);
int cmtj_batch_variants_l2(const CmtjBatchVariant **out);
int cmtj_batch_variants_l3(const CmtjBatchVariant **out);
int cmtj_batch_variants_l4(const CmtjBatchVariant **out);
