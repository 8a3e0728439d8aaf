// FP32 engine: the precision form. FP32 body state, geometry and contact rows with fused
// multiply-adds allowed; accumulated impulses stay in FP64.
#include "pk_engine_host.cuh"

namespace pk
{
EngineBase *make_engine_f32() { return new Engine<float>(); }
} // namespace pk
