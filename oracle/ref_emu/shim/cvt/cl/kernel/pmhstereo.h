/* TEST INFRASTRUCTURE — stand-in for the header the reference's build generates
 * from pmhstereo.cl (cmake/GLCLTOHEADER.cmake); kernels are looked up by name. */
#ifndef CVT_SHIM_pmhstereo_H
#define CVT_SHIM_pmhstereo_H
static const char* _pmhstereo_source = "pmhstereo";
#endif
