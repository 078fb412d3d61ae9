/*
 * TEST INFRASTRUCTURE — stand-in for cvt/cl/CLKernel.h (and CLNDRange /
 * CLLocalSpace / cl_* types): records kernel arguments and runs the kernel of
 * that name in the OpenCL-C emulation.  run() and runWait() both complete the
 * launch before returning.
 */
#ifndef CVT_SHIM_CLKERNEL_H
#define CVT_SHIM_CLKERNEL_H
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include <cvt/gfx/Image.h>
#include <cvt/cl/CLBuffer.h>
#include "clemu_api.h"

typedef int cl_int;
typedef unsigned int cl_uint;
typedef float cl_float;
struct alignas(16) cl_float4 { float s[4]; };
struct alignas(32) cl_float8 { float s[8]; };

namespace cvt {

struct CLLocalSpace {
    CLLocalSpace(size_t s) : size(s) {}
    size_t size;
};

class CLNDRange {
  public:
    CLNDRange() : _dim(0) { _d[0] = _d[1] = _d[2] = 0; }
    CLNDRange(size_t x) : _dim(1) { _d[0] = x; _d[1] = _d[2] = 1; }
    CLNDRange(size_t x, size_t y) : _dim(2) { _d[0] = x; _d[1] = y; _d[2] = 1; }
    CLNDRange(size_t x, size_t y, size_t z) : _dim(3) { _d[0] = x; _d[1] = y; _d[2] = z; }
    size_t operator[](int i) const { return _d[i]; }
    size_t dimension() const { return _dim; }
  private:
    size_t _d[3];
    size_t _dim;
};

inline clemu::Arg cl_arg(int v) { clemu::Arg a; a.kind = clemu::Arg::INT; a.i = v; return a; }
inline clemu::Arg cl_arg(float v) { clemu::Arg a; a.kind = clemu::Arg::FLOAT; a.f = v; return a; }
inline clemu::Arg cl_arg(const cl_float4& v) {
    clemu::Arg a; a.kind = clemu::Arg::FLOAT4;
    for (int i = 0; i < 4; ++i) a.f4[i] = v.s[i];
    return a;
}
inline clemu::Arg cl_arg(const CLLocalSpace& s) { clemu::Arg a; a.kind = clemu::Arg::LOCAL; a.local_size = s.size; return a; }

class CLKernel {
  public:
    CLKernel(const char* source, const char* name) : _name(name) { (void)source; }
    void setArg(cl_uint i, Image& img) const { at(i).kind = clemu::Arg::IMAGE; at(i).img = img.cl(); }
    void setArg(cl_uint i, const Image& img) const { at(i).kind = clemu::Arg::IMAGE; at(i).img = img.cl(); }
    void setArg(cl_uint i, CLBuffer& b) const { at(i).kind = clemu::Arg::BUFFER; at(i).ptr = b.ptr(); }
    void setArg(cl_uint i, const CLBuffer& b) const { at(i).kind = clemu::Arg::BUFFER; at(i).ptr = b.ptr(); }
    template <typename T> void setArg(cl_uint i, T arg) const { at(i) = cl_arg(arg); }
    void run(const CLNDRange& global, const CLNDRange& local, const CLNDRange& offset = CLNDRange()) const {
        (void)offset;
        clemu::launch(_name, _args, global[0], global[1], local[0], local[1]);
    }
    void runWait(const CLNDRange& global, const CLNDRange& local, const CLNDRange& offset = CLNDRange()) const {
        run(global, local, offset);
    }
  private:
    clemu::Arg& at(cl_uint i) const { if (_args.size() <= i) _args.resize(i + 1); return _args[i]; }
    std::string _name;
    mutable std::vector<clemu::Arg> _args;
};

}  // namespace cvt
#endif
