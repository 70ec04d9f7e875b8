// Test stub of the small part of XLA's FFI API (xla/ffi/api/ffi.h, shipped by
// jaxlib) that galax_gb300/xla/gb300_xla.cc uses. jaxlib is not installed on
// the machines that run the CPU tests, so the handler source is compiled
// against this stub instead: the C++ compiler then checks every gal_* call in
// the handlers against include/galax_gb300.h, and XLA_FFI_DEFINE_HANDLER_SYMBOL
// checks that each handler's parameters are exactly what its binding declares
// (context, then arguments, results and attributes, in order). The stub runs
// nothing.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <string_view>
#include <type_traits>

namespace xla::ffi {

enum class DataType : uint8_t { S32, S64, U8, F32, F64 };
inline constexpr DataType S32 = DataType::S32;
inline constexpr DataType S64 = DataType::S64;
inline constexpr DataType U8 = DataType::U8;
inline constexpr DataType F32 = DataType::F32;
inline constexpr DataType F64 = DataType::F64;

template <DataType d> struct Native;
template <> struct Native<DataType::S32> { using type = int32_t; };
template <> struct Native<DataType::S64> { using type = int64_t; };
template <> struct Native<DataType::U8> { using type = uint8_t; };
template <> struct Native<DataType::F32> { using type = float; };
template <> struct Native<DataType::F64> { using type = double; };

template <DataType dtype>
class Buffer {
 public:
  using T = typename Native<dtype>::type;
  T* typed_data() const { return nullptr; }
  void* untyped_data() const { return nullptr; }
  size_t element_count() const { return 0; }
  size_t size_bytes() const { return 0; }
};

template <typename B>
class Result {
 public:
  B* operator->() const { return nullptr; }
};

template <DataType dtype>
using ResultBuffer = Result<Buffer<dtype>>;

class Error {
 public:
  static Error Success() { return Error(); }
  static Error Internal(std::string) { return Error(); }
  static Error InvalidArgument(std::string) { return Error(); }
};

template <typename T> struct PlatformStream {};

namespace stub {
template <typename T> struct CtxTag;
template <typename T> struct CtxTag<PlatformStream<T>> { using param = T; };
template <typename T> struct ArgTag { using param = T; };
template <typename T> struct RetTag;
template <DataType d> struct RetTag<Buffer<d>> { using param = Result<Buffer<d>>; };
template <typename T> struct AttrTag { using param = T; };
}  // namespace stub

template <typename... Tags>
struct Binding {
  template <typename T> Binding<Tags..., stub::CtxTag<T>> Ctx() const { return {}; }
  template <typename T> Binding<Tags..., stub::ArgTag<T>> Arg() const { return {}; }
  template <typename T> Binding<Tags..., stub::RetTag<T>> Ret() const { return {}; }
  template <typename T> Binding<Tags..., stub::AttrTag<T>> Attr(std::string_view) const { return {}; }
  template <typename F> int To(F) const {
    static_assert(std::is_same_v<F, Error (*)(typename Tags::param...)>,
                  "handler parameters differ from its binding");
    return 0;
  }
};

struct Ffi {
  static Binding<> Bind() { return {}; }
};

}  // namespace xla::ffi

#define XLA_FFI_DEFINE_HANDLER_SYMBOL(fn, impl, binding) \
  extern "C" int fn() { return (binding).To(&impl); }
