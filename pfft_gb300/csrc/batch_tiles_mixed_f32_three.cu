// Tile unit of the batched persistent launch (batch_kernel.cuh): mixed-radix
// tiles, FP32, lengths 24, 48, 96, 192, 384, 768.
#include "batch_kernel.cuh"

namespace pg {

PG_BT_DEF_MX(F32, 24)
PG_BT_DEF_MX(F32, 48)
PG_BT_DEF_MX(F32, 96)
PG_BT_DEF_MX(F32, 192)
PG_BT_DEF_MX(F32, 384)
PG_BT_DEF_MX(F32, 768)

}  // namespace pg
