/* TEST INFRASTRUCTURE — stand-in for the header the reference's build generates
 * from PDHuberWeightedInpaint.cl (cmake/GLCLTOHEADER.cmake); kernels are looked up by name. */
#ifndef CVT_SHIM_PDHuberWeightedInpaint_H
#define CVT_SHIM_PDHuberWeightedInpaint_H
static const char* _PDHuberWeightedInpaint_source = "PDHuberWeightedInpaint";
#endif
