// FP64 instantiation of the explicit-MPM engine (2x4x4 SPGrid blocks).
#include "engine_host.cuh"
namespace zr {
std::unique_ptr<EngineBase> make_engine_f64() { return std::unique_ptr<EngineBase>(new Engine<double>()); }
} // namespace zr
