// Stand-in for ParMooN's ErrThrow (include/General/MooNMD_Io.h:210): throws
// std::runtime_error with the arguments concatenated. Test infrastructure
// (see ParameterDatabase.h).
#pragma once
#include <sstream>
#include <stdexcept>

template <class... T>
[[noreturn]] void standin_err_throw(const T&... args) {
  std::ostringstream os;
  (void)std::initializer_list<int>{(os << args, 0)...};
  throw std::runtime_error(os.str());
}
#define ErrThrow(...) standin_err_throw(__VA_ARGS__)
