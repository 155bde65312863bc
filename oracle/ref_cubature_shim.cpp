// Test-only shim over HyperFox's own Cubature class (src/element/Cubature.cpp),
// compiled from the reference sources in place into oracle/_ref/ by
// oracle/build_ref.sh. It lets the CPU tests compare the cubature tables used
// by the oracle and by the CUDA path with the reference's own code.
#include <algorithm>
#include "Cubature.h"

extern "C" int ref_cubature(int dim, int order, int orthotope, double* coords,
                            double* weights, int cap) {
  try {
    hfox::Cubature cub(dim, order, orthotope ? hfox::orthotope : hfox::simplex);
    int n = cub.getNumIPs();
    if (n > cap) return -n;
    const auto* ips = cub.getIPCoords();
    const auto* ws = cub.getIPWeights();
    for (int i = 0; i < n; ++i) {
      for (int k = 0; k < dim; ++k) coords[i * dim + k] = (*ips)[i][k];
      weights[i] = (*ws)[i];
    }
    return n;
  } catch (...) {
    return -1000000;
  }
}
