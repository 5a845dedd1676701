// Test infrastructure only: the few absl::Status names the reference's CUDA
// rasterizer (diffren/common/kernels/rasterize_triangles_impl_cuda.cu.{h,cc})
// uses, so that it compiles without abseil. A status is ok or carries a
// message.
#pragma once
#include <string>
#include <utility>

namespace absl {

class Status {
 public:
  Status() = default;
  explicit Status(std::string message) : ok_(false), message_(std::move(message)) {}
  bool ok() const { return ok_; }
  const std::string& message() const { return message_; }

 private:
  bool ok_ = true;
  std::string message_;
};

inline Status OkStatus() { return Status(); }
inline Status UnknownError(const std::string& message) { return Status(message); }

}  // namespace absl
