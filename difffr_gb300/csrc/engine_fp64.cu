// Engine<double>: FP64 fluid arithmetic (the reference's USE_DOUBLE build).
#include "engine_impl.cuh"

namespace dfsph {
template class Engine<double>;
EngineBase *make_engine_fp64(const dfsph_scene *sc) { return new Engine<double>(sc); }
}  // namespace dfsph
