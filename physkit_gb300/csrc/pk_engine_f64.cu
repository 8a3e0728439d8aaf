// FP64 engine: the parity form. Built with -fmad=false so every multiply and add rounds as
// written, which makes its results identical to the FP64 CPU oracle run in the same solver order.
#include "pk_engine_host.cuh"

namespace pk
{
EngineBase *make_engine_f64() { return new Engine<double>(); }
} // namespace pk
