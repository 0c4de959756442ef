// FP64 engine.
#include "engine_impl.cuh"

namespace glia {
EngineBase* make_engine_f64(int n, bool reference_structured) {
  return new Engine<double>(n, reference_structured);
}
}  // namespace glia
