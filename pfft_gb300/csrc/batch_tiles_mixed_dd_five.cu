// Tile unit of the batched persistent launch (batch_kernel.cuh): mixed-radix
// tiles, float-float, lengths 40, 80, 160, 320, 640.
#include "batch_kernel.cuh"

namespace pg {

PG_BT_DEF_MX(FDD, 40)
PG_BT_DEF_MX(FDD, 80)
PG_BT_DEF_MX(FDD, 160)
PG_BT_DEF_MX(FDD, 320)
PG_BT_DEF_MX(FDD, 640)

}  // namespace pg
