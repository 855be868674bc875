// FP64 iterates: instantiates the engine for double.
#include "engine_impl.cuh"

namespace sps {
EngineBase* make_engine_f64() { return new Engine<double>(); }
int setup_f64(EngineBase* e, const HostProblem& hp, const sps_options& o, int mode) {
    return static_cast<Engine<double>*>(e)->setup(hp, o, mode);
}
}  // namespace sps
