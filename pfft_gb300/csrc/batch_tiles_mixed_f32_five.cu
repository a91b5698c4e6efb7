// Tile unit of the batched persistent launch (batch_kernel.cuh): mixed-radix
// tiles, FP32, lengths 40, 80, 160, 320, 640.
#include "batch_kernel.cuh"

namespace pg {

PG_BT_DEF_MX(F32, 40)
PG_BT_DEF_MX(F32, 80)
PG_BT_DEF_MX(F32, 160)
PG_BT_DEF_MX(F32, 320)
PG_BT_DEF_MX(F32, 640)

}  // namespace pg
