// Tile unit of the batched persistent launch (batch_kernel.cuh): mixed-radix
// tiles, float-float, lengths 24, 48, 96, 192, 384, 768.
#include "batch_kernel.cuh"

namespace pg {

PG_BT_DEF_MX(FDD, 24)
PG_BT_DEF_MX(FDD, 48)
PG_BT_DEF_MX(FDD, 96)
PG_BT_DEF_MX(FDD, 192)
PG_BT_DEF_MX(FDD, 384)
PG_BT_DEF_MX(FDD, 768)

}  // namespace pg
