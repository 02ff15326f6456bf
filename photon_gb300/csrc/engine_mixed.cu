// Mixed-precision instantiation of the engine: FP32 fields and stencils
// (multiply-adds fused), the pressure solve as FP32 multigrid CG inside an
// FP64 refinement loop, FP64 dot products and global sums.
#include "engine.cuh"

namespace phx {

CtxBase* makeCtxMixed() { return new Ctx<float>(); }

}  // namespace phx
