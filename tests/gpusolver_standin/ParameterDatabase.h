// Stand-in for ParMooN's ParameterDatabase (include/General/ParameterDatabase.h)
// with the one member GpuSolver uses: write(std::ostream&, bool), in the
// reference's non-verbose format ("[ name ]", then "key: value" lines).
// Test infrastructure: lets tests/test_gpu_integration.py compile
// integration/GpuSolver.C on a machine without the reference sources.
#pragma once
#include <ostream>
#include <string>
#include <utility>
#include <vector>

class ParameterDatabase {
 public:
  explicit ParameterDatabase(std::string name) : name_(std::move(name)) {}
  void set(const std::string& k, const std::string& v) {
    for (auto& kv : kv_)
      if (kv.first == k) { kv.second = v; return; }
    kv_.emplace_back(k, v);
  }
  void write(std::ostream& os, bool = false) const {
    os << "# A ParMooN parameter database with " << kv_.size() << " parameters and 0 nested databases\n\n";
    os << "[ " << name_ << " ]\n\n";
    for (const auto& kv : kv_) os << kv.first << ": " << kv.second << "\n";
  }
 private:
  std::string name_;
  std::vector<std::pair<std::string, std::string>> kv_;
};
