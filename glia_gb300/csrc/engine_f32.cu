// Mixed-precision engine: float fields and transforms, FP64 reductions and scalars.
#include "engine_impl.cuh"

namespace glia {
EngineBase* make_engine_f32(int n, bool reference_structured) {
  return new Engine<float>(n, reference_structured);
}
}  // namespace glia
