/* TEST INFRASTRUCTURE — force-included into the reference's
 * PMHuberStereo.cpp: provides std::cout and makes the debug block's
 * getchar() (PMHuberStereo.cpp:184) return at once instead of waiting on a
 * terminal.  It changes no result. */
#include <cstdio>
#include <iostream>
#undef getchar
#define getchar() (0)
