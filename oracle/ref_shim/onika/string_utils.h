#pragma once
#include <cstdio>
#include <string>
#include <vector>
// Stand-in: onika::format_string, printf-style formatting into a std::string
// (std::string arguments are passed as C strings).
namespace onika {
namespace detail {
template <class T>
inline T fmt_arg(const T& v) { return v; }
inline const char* fmt_arg(const std::string& s) { return s.c_str(); }
}  // namespace detail
template <class... Args>
inline std::string format_string(const std::string& fmt, const Args&... args) {
  const int len = std::snprintf(nullptr, 0, fmt.c_str(), detail::fmt_arg(args)...);
  if (len <= 0) return std::string();
  std::vector<char> buf((size_t)len + 1);
  std::snprintf(buf.data(), buf.size(), fmt.c_str(), detail::fmt_arg(args)...);
  return std::string(buf.data(), (size_t)len);
}
}  // namespace onika
