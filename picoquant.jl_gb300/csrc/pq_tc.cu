// Split-precision tensor-core contraction class (tcgen05).  Shapes that are
// not eligible fall back to the SIMT GEMM class at analysis time.
#include "pq_internal.h"

namespace pq {

bool tc_eligible(int precision, const GemmDesc& d) {
  (void)precision;
  (void)d;
  return false;
}

size_t tc_scratch_bytes(int precision, const GemmDesc& d) {
  (void)precision;
  (void)d;
  return 0;
}

cudaError_t launch_tc(int precision, int ta, int tb, int tc, const void* A, const void* B, void* C,
                      const GemmDesc& d, void* scratch, size_t scratch_bytes, cudaStream_t stream) {
  (void)precision;
  (void)ta;
  (void)tb;
  (void)tc;
  (void)A;
  (void)B;
  (void)C;
  (void)d;
  (void)scratch;
  (void)scratch_bytes;
  (void)stream;
  return cudaErrorNotSupported;
}

}  // namespace pq
