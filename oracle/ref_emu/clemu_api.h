/*
 * clemu_api.h — TEST INFRASTRUCTURE.  The part of the OpenCL-C emulation that
 * host-side code (the shims the reference's PMHuberStereo.cpp and PDROF.h
 * compile against, and the harness) may include: images, kernel arguments and
 * launches by kernel name.  No OpenCL vocabulary macros here.
 */
#ifndef CLEMU_API_H
#define CLEMU_API_H

#include <cstddef>
#include <functional>
#include <string>
#include <vector>

namespace clemu {

struct Img {
    int w, h;
    int channels;     /* 4: CL_RGBA/CL_FLOAT, 2: CL_RG/CL_FLOAT, 1: CL_INTENSITY/CL_FLOAT */
    float* data;
};

struct Arg {
    enum Kind { NONE, IMAGE, BUFFER, INT, FLOAT, FLOAT4, LOCAL, BYTES } kind = NONE;
    Img* img = nullptr;
    void* ptr = nullptr;
    int i = 0;
    float f = 0.0f;
    float f4[4] = {0, 0, 0, 0};
    size_t local_size = 0;
    std::vector<unsigned char> bytes;   /* BYTES: a struct passed by value (clSetKernelArg with its size) */
};

/* Runs kernel `name` over a 2-D NDRange (global gx x gy, local lx x ly). */
void launch(const std::string& name, const std::vector<Arg>& args, size_t gx, size_t gy, size_t lx, size_t ly);
/* The same over a 3-D NDRange with local size lx x ly x 1. */
void launch3(const std::string& name, const std::vector<Arg>& args, size_t gx, size_t gy, size_t gz, size_t lx,
             size_t ly);
bool has_kernel(const std::string& name);

/* Called after every launch with the kernel name and its arguments. */
extern std::function<void(const std::string&, const std::vector<Arg>&)> on_launch;

/* patch_eval_color_grad_weighted of pmhstereo.cl, called directly. */
float pmh_patch_eval(Img* col1, Img* grad1, Img* col2, Img* grad2, float cx, float cy, const float state[4],
                     int patchsize, int lr);

}  // namespace clemu

#endif
