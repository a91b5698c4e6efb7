// Tile unit of the batched persistent launch (batch_kernel.cuh): mixed-radix
// tiles, 64-bit fixed point (FX), lengths 40, 80, 160, 320, 640.
#include "batch_kernel.cuh"

namespace pg {

PG_BT_DEF_MX(FX, 40)
PG_BT_DEF_MX(FX, 80)
PG_BT_DEF_MX(FX, 160)
PG_BT_DEF_MX(FX, 320)
PG_BT_DEF_MX(FX, 640)

}  // namespace pg
