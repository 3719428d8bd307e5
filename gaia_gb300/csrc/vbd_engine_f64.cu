// The StF64 engine (vbd_engine.cuh), compiled on its own so that the precision modes build in
// parallel.
#include "vbd_engine.cuh"

namespace gaia {
EngineBase* make_engine_f64(const Scene& s, int mode) { return new Engine<dev::StF64, double>(s, mode); }
}  // namespace gaia
