// Tile unit of the batched persistent launch (batch_kernel.cuh): general FP64 tiles.
#include "batch_kernel.cuh"

namespace pg {

PG_BT_DEF_GEN(bt_gen_f64_m, ArF64, -1)
PG_BT_DEF_GEN(bt_gen_f64_p, ArF64, 1)
PG_BT_DEF_SMALL(bt_small_f64_m, ArF64, -1)
PG_BT_DEF_SMALL(bt_small_f64_p, ArF64, 1)

}  // namespace pg
