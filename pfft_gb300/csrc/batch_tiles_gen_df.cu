// Tile unit of the batched persistent launch (batch_kernel.cuh): general float-float tiles.
#include "batch_kernel.cuh"

namespace pg {

PG_BT_DEF_GEN(bt_gen_df_m, ArDF, -1)
PG_BT_DEF_GEN(bt_gen_df_p, ArDF, 1)
PG_BT_DEF_SMALL(bt_small_df_m, ArDF, -1)
PG_BT_DEF_SMALL(bt_small_df_p, ArDF, 1)

}  // namespace pg
