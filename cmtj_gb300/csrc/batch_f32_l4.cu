// FP32 batched kernel variants for junctions with 4 layer(s).
#include "batch_variants.cuh"

static const CmtjBatchVariant kVariants[] = CMTJ_BATCH_VARIANT_TABLE(4);

int cmtj_batch_variants_l4(const CmtjBatchVariant **out) {
  *out = kVariants;
  return (int)(sizeof(kVariants) / sizeof(kVariants[0]));
}
