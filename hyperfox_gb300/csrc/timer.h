// Per-kernel CUDA-event timing on the launching stream (optional, per context).
#pragma once
#include <cuda_runtime.h>

#include <vector>

namespace hfx {

enum KernelId {
  K_LOCAL = 0,      // element assembly + condensation
  K_SCATTER = 1,    // trace CSR scatter (values + rhs)
  K_SPMV64 = 2,     // CG operator application, FP64
  K_SPMV32 = 3,     // CG operator application, FP32 (mixed precision)
  K_UPDATE = 4,     // CG vector update + preconditioner (both precisions)
  K_RECOVER = 5,    // local recovery
  K_OTHER = 6,      // setup kernels of the solve (system prep, preconditioner, residuals)
  K_RESIDUAL = 7,   // FP64 matrix-free residual of the full HDG system (mixed precision)
  K_COARSE = 8,     // two-level preconditioner: restriction, Chebyshev coarse solve, coarse setup
  K_TENSOR = 9,     // element contractions on the tensor cores (tc_assembly.cu)
  K_COUNT = 10
};

class KernelTimer {
 public:
  ~KernelTimer() { reset(); }
  void enable(bool on) { on_ = on; }
  bool enabled() const { return on_; }
  void begin(int id, cudaStream_t s) {
    if (!on_) return;
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, s);
    open_.push_back({id, e});
  }
  void end(int id, cudaStream_t s) {
    if (!on_) return;
    for (size_t i = open_.size(); i-- > 0;)
      if (open_[i].id == id) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        cudaEventRecord(e, s);
        done_.push_back({id, open_[i].e, e});
        open_.erase(open_.begin() + i);
        return;
      }
  }
  // Totals over all recorded launches (synchronises on the events).
  void read(int id, int* launches, double* ms) {
    int n = 0;
    double t = 0.0;
    for (auto& r : done_) {
      if (r.id != id) continue;
      float x = 0.f;
      cudaEventSynchronize(r.e1);
      cudaEventElapsedTime(&x, r.e0, r.e1);
      t += x;
      ++n;
    }
    *launches = n;
    *ms = t;
  }
  void reset() {
    for (auto& r : done_) {
      cudaEventDestroy(r.e0);
      cudaEventDestroy(r.e1);
    }
    for (auto& o : open_) cudaEventDestroy(o.e);
    done_.clear();
    open_.clear();
  }

 private:
  struct Open {
    int id;
    cudaEvent_t e;
  };
  struct Rec {
    int id;
    cudaEvent_t e0, e1;
  };
  bool on_ = false;
  std::vector<Open> open_;
  std::vector<Rec> done_;
};

}  // namespace hfx
