/* TEST INFRASTRUCTURE — stand-in for cvt/util/Exception.h. */
#ifndef CVT_SHIM_EXCEPTION_H
#define CVT_SHIM_EXCEPTION_H
#include <stdexcept>
#include <string>
namespace cvt {
class CVTException : public std::runtime_error {
  public:
    CVTException(const char* m) : std::runtime_error(m) {}
    CVTException(const std::string& m) : std::runtime_error(m) {}
};
}
#endif
