/* TEST INFRASTRUCTURE — stand-in for the header the reference's build generates
 * from fill.cl (cmake/GLCLTOHEADER.cmake); kernels are looked up by name. */
#ifndef CVT_SHIM_fill_H
#define CVT_SHIM_fill_H
static const char* _fill_source = "fill";
#endif
