// Stand-in for ParMooN's TMatrix (include/Matrix/Matrix.h): CSR arrays with
// the reference's accessor names. Test infrastructure (see ParameterDatabase.h).
#pragma once
#include <vector>

class TMatrix {
 public:
  TMatrix(int n_rows, int n_cols, std::vector<int> rows, std::vector<int> cols, std::vector<double> vals)
      : nr(n_rows), nc(n_cols), rp(std::move(rows)), ci(std::move(cols)), v(std::move(vals)) {}
  int GetN_Rows() const { return nr; }
  int GetN_Columns() const { return nc; }
  const int* GetRowPtr() const { return rp.data(); }
  const int* GetKCol() const { return ci.data(); }
  const double* GetEntries() const { return v.data(); }
 private:
  int nr, nc;
  std::vector<int> rp, ci;
  std::vector<double> v;
};
