// cvo_irls.cu -- multi-frame RKHS-BA (CvoBatchIRLS::solve, src/cvo/IRLS.cpp:148-367).
#include "cvo_internal.h"

namespace cvo_gb {

int run_align_multi(Handle *h, int n_frames, DevCloud *const *clouds, double *poses, const uint8_t *hold_const,
                    int n_edges, const int *edges, double *secs, int *iters) {
  (void)h; (void)n_frames; (void)clouds; (void)poses; (void)hold_const; (void)n_edges; (void)edges;
  (void)secs; (void)iters;
  return CVO_ERR_UNSUPPORTED;
}

}  // namespace cvo_gb
