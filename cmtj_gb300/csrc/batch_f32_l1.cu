// FP32 batched kernel variants for junctions with 1 layer(s).
#include "batch_variants.cuh"

static const CmtjBatchVariant kVariants[] = CMTJ_BATCH_VARIANT_TABLE(1);

int cmtj_batch_variants_l1(const CmtjBatchVariant **out) {
  *out = kVariants;
  return (int)(sizeof(kVariants) / sizeof(kVariants[0]));
}
