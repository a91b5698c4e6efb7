// Tile unit of the batched persistent launch (batch_kernel.cuh): general FP32 tiles.
#include "batch_kernel.cuh"

namespace pg {

PG_BT_DEF_GEN(bt_gen_f32_m, ArF32, -1)
PG_BT_DEF_GEN(bt_gen_f32_p, ArF32, 1)
PG_BT_DEF_SMALL(bt_small_f32_m, ArF32, -1)
PG_BT_DEF_SMALL(bt_small_f32_p, ArF32, 1)

}  // namespace pg
