// engine_fp32.cu - kernel instantiations with float population storage.
#include "engine_impl.cuh"

namespace pflbm {
Engine *make_engine_fp32(int q, bool jet, const HostParams &hp, uint32_t flags) {
    return make_engine_t<float>(q, jet, hp, flags);
}
}  // namespace pflbm
