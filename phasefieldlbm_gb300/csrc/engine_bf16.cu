// engine_bf16.cu - kernel instantiations with __nv_bfloat16 population storage.
#include "engine_impl.cuh"

namespace pflbm {
Engine *make_engine_bf16(int q, bool jet, const HostParams &hp, uint32_t flags) {
    return make_engine_t<__nv_bfloat16>(q, jet, hp, flags);
}
}  // namespace pflbm
