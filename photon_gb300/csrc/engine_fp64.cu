// FP64 instantiation of the engine: every field and every operation in double
// precision. Built with --fmad=false so that no multiply and add are fused, as
// in the reference's own arithmetic.
#include "engine.cuh"

namespace phx {

CtxBase* makeCtxFp64() { return new Ctx<double>(); }

}  // namespace phx
