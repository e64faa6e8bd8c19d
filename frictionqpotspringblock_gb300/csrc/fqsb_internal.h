/*
 * Internal host-side interface between the C-ABI layer (fqsb_capi.cu) and the
 * kernel translation units.  Not installed; the public ABI is include/fqsb.h.
 */
#ifndef FQSB_INTERNAL_H
#define FQSB_INTERNAL_H

#include <cuda_runtime.h>

#include <string>

#include "fqsb_device.cuh"

namespace fqsb {

/* Launch geometry of the 1d step kernel: threads per CTA and particles per thread. */
struct LineGeom {
    int threads;
    int ppt;
    int64_t grid;
};

LineGeom line_geometry(int64_t N);

/* Message returned by fqsb_last_error(NULL) (errors of calls that have no handle). */
void set_global_error(const std::string& msg);

/* Per-particle canonical reduction of the step's residual terms (used by the 2d path). */
int64_t grid_reduce_ctas(int64_t N);

/* Number of CTAs of the step kernel (size of DevSys::cta_pending and DevSys::partials). */
int64_t step_ctas(const DevSys& s, const LineGeom& g);

/* The run graph: a device-side WHILE loop over fused steps, with the chunk-regeneration branch.
 * Writes the conditional handles into s (they are kernel arguments of the graph's nodes). */
cudaError_t build_run_graph(DevSys& s, const LineGeom& g, cudaGraphExec_t* exec);

} // namespace fqsb

#endif
