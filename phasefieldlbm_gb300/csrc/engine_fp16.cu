// engine_fp16.cu - kernel instantiations with __half population storage.
#include "engine_impl.cuh"

namespace pflbm {
Engine *make_engine_fp16(int q, bool jet, const HostParams &hp, uint32_t flags) {
    return make_engine_t<__half>(q, jet, hp, flags);
}
}  // namespace pflbm
