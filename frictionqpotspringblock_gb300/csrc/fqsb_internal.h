/*
 * Internal host-side interface between the C-ABI layer (fqsb_capi.cu) and the
 * kernel translation units.  Not installed; the public ABI is include/fqsb.h.
 */
#ifndef FQSB_INTERNAL_H
#define FQSB_INTERNAL_H

#include <cuda_runtime.h>

#include "fqsb_device.cuh"

namespace fqsb {

/* Launch geometry of the 1d step kernel: threads per CTA and particles per thread. */
struct LineGeom {
    int threads;
    int ppt;
    int64_t grid;
};

LineGeom line_geometry(int64_t N);

/* One velocity-Verlet step of a Line1d / Particles system (finalises the step itself). */
cudaError_t launch_step_line(const DevSys& s, const LineGeom& g, bool units, cudaStream_t st);

/* One step of a Line2d system: step kernel + reduction/finalise kernel. */
cudaError_t launch_step_grid(const DevSys& s, bool units, cudaStream_t st);

/* Per-particle canonical reduction of the step's residual terms (used by the 2d path). */
int64_t grid_reduce_ctas(int64_t N);

} // namespace fqsb

#endif
