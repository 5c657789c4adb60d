// FP32 instantiation of the explicit-MPM engine (4x4x4 SPGrid blocks).
#include "engine_host.cuh"
namespace zr {
std::unique_ptr<EngineBase> make_engine_f32() { return std::unique_ptr<EngineBase>(new Engine<float>()); }
} // namespace zr
