// Learned preconditioner entry points (network kernels live in cnn.cu once loaded).
#include "ctx.h"

namespace gbc {
void precond_free(gbc_ctx* c) {
  if (!c) return;
  c->precond = nullptr;
}
void precond_apply(gbc_ctx* c, const Spinor& in, const Spinor& out) { blas_copy(c->g, out, in, c->stream); }
}  // namespace gbc

extern "C" int gbc_load_precond(gbc_ctx* c, const char* path) {
  if (!c || !path) return GBC_ERR_ARGS;
  c->err = "learned preconditioner not available in this build";
  return GBC_ERR_PRECOND;
}
