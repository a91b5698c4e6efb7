// Tile unit of the batched persistent launch (batch_kernel.cuh): mixed-radix
// tiles, block-quantised float-float, lengths 40, 80, 160, 320, 640.
#include "batch_kernel.cuh"

namespace pg {

PG_BT_DEF_MX(FQ, 40)
PG_BT_DEF_MX(FQ, 80)
PG_BT_DEF_MX(FQ, 160)
PG_BT_DEF_MX(FQ, 320)
PG_BT_DEF_MX(FQ, 640)

}  // namespace pg
