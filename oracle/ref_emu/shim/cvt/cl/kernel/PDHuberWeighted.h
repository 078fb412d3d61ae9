/* TEST INFRASTRUCTURE — stand-in for the header the reference's build generates
 * from PDHuberWeighted.cl (cmake/GLCLTOHEADER.cmake); kernels are looked up by name. */
#ifndef CVT_SHIM_PDHuberWeighted_H
#define CVT_SHIM_PDHuberWeighted_H
static const char* _PDHuberWeighted_source = "PDHuberWeighted";
#endif
