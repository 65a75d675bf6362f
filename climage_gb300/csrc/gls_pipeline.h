// gls_pipeline.h -- internals of the RawConverter pipeline shared between translation units.
#ifndef GLS_PIPELINE_H
#define GLS_PIPELINE_H

#include "gls_internal.h"

namespace gls {

void host_cam_ycbcr(const float rgb_cam[9], float out[9]);
bool host_inverse3x3(const float m[9], float out[9]);

}  // namespace gls

#endif  // GLS_PIPELINE_H
