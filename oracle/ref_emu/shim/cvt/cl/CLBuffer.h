/* TEST INFRASTRUCTURE — stand-in for cvt/cl/CLBuffer.h: zero-filled host memory. */
#ifndef CVT_SHIM_CLBUFFER_H
#define CVT_SHIM_CLBUFFER_H
#include <cstddef>
#include <cstdint>
#include <vector>
namespace cvt {
class CLBuffer {
  public:
    explicit CLBuffer(size_t size) : _mem((size + 15) / 16 * 16 + 16, 0) {}
    void* ptr() const { return (void*)(((uintptr_t)_mem.data() + 15) & ~(uintptr_t)15); }
    size_t size() const { return _mem.size() - 16; }
  private:
    std::vector<char> _mem;
};
}
#endif
