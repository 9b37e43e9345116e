// Generalized winding number sign for non-watertight meshes.
#include "api_internal.h"

sdfb_status gwn_apply(sdfb_ctx *ctx, cudaStream_t, const sdfb::MeshDev &, const BakeInput &, const sdfb_grid_desc &,
                      const sdfb_opts &, float *, uint32_t *) {
  return ctx_fail(ctx, SDFB_ERR_INTERNAL, "winding-number sign is not available in this build");
}
