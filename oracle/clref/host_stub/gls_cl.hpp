// gls_cl.hpp (stand-in): nothing of the OpenCL runtime is needed where this directory is on
// the include path (see gls_cl_image.hpp).  TEST INFRASTRUCTURE ONLY.
#ifndef GLS_CL_STUB_HPP
#define GLS_CL_STUB_HPP
#include "gls_cl_image.hpp"
#endif
