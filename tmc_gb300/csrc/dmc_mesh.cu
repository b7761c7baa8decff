#include "../../include/tmc_gb300.h"
#include "dmc_mesh.h"

namespace tmc {

DmcPostStatus dmc_postprocess(const DmcMesh& in, uint32_t flags, int sms, cudaStream_t st, DmcPostOut* out) {
  (void)sms;
  (void)st;
  DmcPostStatus s;
  out->mesh = in;
  if (flags & (TMC_DMC_P3X3Y_COLOR | TMC_DMC_P3X3Y_ISOLATED | TMC_DMC_P3333 | TMC_OUT_TRIANGLES | TMC_OUT_HALFEDGES))
    s.err = cudaErrorNotSupported;
  return s;
}

}  // namespace tmc
