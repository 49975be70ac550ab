// Mixed-precision pass (placeholder until the FP32 floatexp kernel lands).
#include "engine.h"

namespace mbx {
cudaError_t Engine::run_mixed_pass(const DeviceFrame&) { return cudaErrorNotSupported; }
int Engine::prepare_mixed() { return MBX_OK; }
} // namespace mbx
