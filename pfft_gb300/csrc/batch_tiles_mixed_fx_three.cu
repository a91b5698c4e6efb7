// Tile unit of the batched persistent launch (batch_kernel.cuh): mixed-radix
// tiles, 64-bit fixed point (FX), lengths 24, 48, 96, 192, 384, 768.
#include "batch_kernel.cuh"

namespace pg {

PG_BT_DEF_MX(FX, 24)
PG_BT_DEF_MX(FX, 48)
PG_BT_DEF_MX(FX, 96)
PG_BT_DEF_MX(FX, 192)
PG_BT_DEF_MX(FX, 384)
PG_BT_DEF_MX(FX, 768)

}  // namespace pg
