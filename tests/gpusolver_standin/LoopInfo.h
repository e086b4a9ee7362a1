// Stand-in for ParMooN's LoopInfo (include/General/LoopInfo.h): restart,
// finish and the three getters, with the reference's bookkeeping
// (src/General/LoopInfo.C: finish adds the loop's iterations to the count).
// Test infrastructure (see ParameterDatabase.h).
#pragma once
#include <string>

class LoopInfo {
 public:
  explicit LoopInfo(const std::string& n) : name(n) {}
  void restart(const std::string& n, double initial) {
    name = n;
    initial_residual = initial;
  }
  void finish(unsigned loop_index, double current) {
    n_previous_iterations += loop_index;
    old_residual = current;
  }
  double get_initial_residual() const { return initial_residual; }
  double get_previous_residual() const { return old_residual; }
  unsigned get_n_previous_iterations() const { return n_previous_iterations; }
 private:
  std::string name;
  double initial_residual = 0.0, old_residual = 0.0;
  unsigned n_previous_iterations = 0;
};
