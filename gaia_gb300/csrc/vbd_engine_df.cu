// The StDF engine (vbd_engine.cuh), compiled on its own so that the precision modes build in
// parallel.
#include "vbd_engine.cuh"

namespace gaia {
EngineBase* make_engine_df(const Scene& s, int mode) { return new Engine<dev::StDF, float>(s, mode); }
}  // namespace gaia
