// Split-precision (BF16x3) tensor-core local operator -- placeholder until the
// tcgen05 kernels land; the entry points report TTG_ERR_UNSUPPORTED.
#include "ttg_davidson.cuh"

namespace ttg {

size_t split_matvec_bytes(const LocalDims&, int) { return 0; }

void split_matvec_factory(const LocalDims&, const double*, const double*, const double*, int,
                          void*, cudaStream_t, MatvecFn*) {
  throw Error{TTG_ERR_UNSUPPORTED, "split-precision matvec not built"};
}

}  // namespace ttg

extern "C" int ttg_dbfun3_split(ttg_ctx* ctx, ttg_int, ttg_int, ttg_int, ttg_int, ttg_int,
                                ttg_int, ttg_int, ttg_int, const double*, const double*,
                                const double*, const double*, double*, ttg_int) {
  if (!ctx) return TTG_ERR_ARG;
  ctx->last_error = "split-precision matvec not built";
  return TTG_ERR_UNSUPPORTED;
}
