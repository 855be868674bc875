// FP32 iterates: instantiates the engine for float.
#include "engine_impl.cuh"

namespace sps {
EngineBase* make_engine_f32() { return new Engine<float>(); }
int setup_f32(EngineBase* e, const HostProblem& hp, const sps_options& o, int mode) {
    return static_cast<Engine<float>*>(e)->setup(hp, o, mode);
}
}  // namespace sps
