// cuda::BarnesHut (placeholder until the tree path lands).
#include "pt_common.cuh"

void pt_bh_state_free(pt_ctx *ctx) { (void)ctx; }
