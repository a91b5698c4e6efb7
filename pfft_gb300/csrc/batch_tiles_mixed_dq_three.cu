// Tile unit of the batched persistent launch (batch_kernel.cuh): mixed-radix
// tiles, block-quantised float-float, lengths 24, 48, 96, 192, 384, 768.
#include "batch_kernel.cuh"

namespace pg {

PG_BT_DEF_MX(FQ, 24)
PG_BT_DEF_MX(FQ, 48)
PG_BT_DEF_MX(FQ, 96)
PG_BT_DEF_MX(FQ, 192)
PG_BT_DEF_MX(FQ, 384)
PG_BT_DEF_MX(FQ, 768)

}  // namespace pg
