// Mixed-precision instantiation of the scenario context: FP32 fields and
// stencils (multiply-adds fused), the pressure solve as FP32 multigrid CG
// inside an FP64 refinement loop, FP64 dot products and global sums.
#include "engine.cuh"

namespace phx {

CtxBase* makeCtxMixed(const phx_grid* g, std::string& err) {
    auto* c = new Ctx<float>();
    int r = c->init(g);
    if (r != PHX_OK) {
        err = c->err;
        delete c;
        return nullptr;
    }
    return c;
}

}  // namespace phx
