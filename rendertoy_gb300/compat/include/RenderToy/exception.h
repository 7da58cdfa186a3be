// RenderToy/exception.h — (RenderToy include/RenderToy/exception.h:6-20),
// plus the error raised when the GPU library reports a failure.
#ifndef RTX_COMPAT_EXCEPTION_H
#define RTX_COMPAT_EXCEPTION_H
#include <stdexcept>
#include <string>

namespace RenderToy::Exception {
struct IRenderToyException : public std::runtime_error {
  explicit IRenderToyException(const std::string& m) : std::runtime_error(m) {}
};
struct ImageSizeNotMatchException : public IRenderToyException {
  explicit ImageSizeNotMatchException(const std::string& m) : IRenderToyException(m) {}
};
// A librtx call failed (status code and rtx_last_error message)
struct DeviceException : public IRenderToyException {
  int code;
  DeviceException(int code_, const std::string& m) : IRenderToyException(m), code(code_) {}
};
}  // namespace RenderToy::Exception
#endif
