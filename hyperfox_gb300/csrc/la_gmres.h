// Generic sparse system behind hfx_la_* (LinAlgebraInterface, LinAlgebraInterface.h:23-162).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <unordered_map>
#include <vector>

namespace hfx {

struct LaSolveResult {
  int iterations = 0;
  double rel_residual = 0.0;
  float ms = 0.f;
};

// Values are accumulated on the host with PETSc's ADD_VALUES / INSERT_VALUES
// semantics (PetscInterface.cpp:116-196); assemble() freezes them into a CSR
// with sorted columns; solve() runs restarted GMRES on the device.
class LaSystem {
 public:
  void allocate(int n);
  bool allocated() const { return n_ > 0; }
  bool assembled() const { return assembled_; }
  bool add_block(int nr, const int* rows, int nc, const int* cols, const double* vals, bool insert,
                 std::string* err);
  bool add_rhs(int n, const int* idx, const double* vals, bool insert, std::string* err);
  bool zero_rows(int n, const int* rows, std::string* err);
  void assemble();
  void clear();
  int64_t nnz() const { return (int64_t)col_.size(); }
  // Returns an HFX status code.
  int solve(double rtol, int maxits, int restart, int jacobi, cudaStream_t s, double* x, LaSolveResult* r,
            std::string* err);

 private:
  int n_ = 0;
  bool assembled_ = false;
  std::vector<std::unordered_map<int, double>> rows_;
  std::vector<double> rhs_;
  std::vector<int64_t> rowptr_;
  std::vector<int> col_;
  std::vector<double> val_;
};

}  // namespace hfx
