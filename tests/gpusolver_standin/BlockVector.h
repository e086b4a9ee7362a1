// Stand-in for ParMooN's BlockVector (include/Matrix/BlockVector.h): one
// contiguous block. Test infrastructure (see ParameterDatabase.h).
#pragma once
#include <vector>

class BlockVector {
 public:
  explicit BlockVector(size_t n) : v(n, 0.0) {}
  unsigned int length() const { return unsigned(v.size()); }
  const double* get_entries() const { return v.data(); }
  double* get_entries() { return v.data(); }
 private:
  std::vector<double> v;
};
