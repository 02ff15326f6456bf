// Mixed-precision scenario context (FP32 fields and stencils, FP16 smoother
// scratch, FP64 dots, residual refinement and global sums).
#include "engine.h"

namespace phx {

CtxBase* makeCtxMixed(const phx_grid*, std::string& err) {
    err = "the mixed-precision context is not implemented yet";
    return nullptr;
}

}  // namespace phx
