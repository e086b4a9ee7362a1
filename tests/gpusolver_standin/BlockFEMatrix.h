// Stand-in for ParMooN's BlockFEMatrix (include/Matrix/BlockFEMatrix.h) of a
// one-block convection-diffusion system: get_combined_matrix, get_n_cell_rows
// and get_row_space(b)->GetN_DegreesOfFreedom / GetActiveBound. Test
// infrastructure (see ParameterDatabase.h).
#pragma once
#include <memory>

#include "Matrix.h"

struct StandInSpace {
  int n_dofs, active;
  int GetN_DegreesOfFreedom() const { return n_dofs; }
  int GetActiveBound() const { return active; }
};

class BlockFEMatrix {
 public:
  BlockFEMatrix(std::shared_ptr<TMatrix> A, int active)
      : A_(std::move(A)), space_(std::make_shared<StandInSpace>(StandInSpace{A_->GetN_Rows(), active})) {}
  std::shared_ptr<TMatrix> get_combined_matrix() const { return A_; }
  size_t get_n_cell_rows() const { return 1; }
  std::shared_ptr<const StandInSpace> get_row_space(size_t) const { return space_; }
 private:
  std::shared_ptr<TMatrix> A_;
  std::shared_ptr<const StandInSpace> space_;
};
