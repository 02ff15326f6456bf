// FP64 instantiation of the scenario context: every field and every operation
// in double precision. Built with --fmad=false so that no multiply and add are
// fused, as in the reference's own arithmetic.
#include "engine.cuh"

namespace phx {

CtxBase* makeCtxFp64(const phx_grid* g, std::string& err) {
    auto* c = new Ctx<double>();
    int r = c->init(g);
    if (r != PHX_OK) {
        err = c->err;
        delete c;
        return nullptr;
    }
    return c;
}

}  // namespace phx
