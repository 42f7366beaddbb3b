// Engine<float>: FP32 fluid arithmetic, FP64 rigid state and reductions.
#include "engine_impl.cuh"

namespace dfsph {
template class Engine<float>;
EngineBase *make_engine_fp32(const dfsph_scene *sc) { return new Engine<float>(sc); }
}  // namespace dfsph
