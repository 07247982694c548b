// engine_fp64.cu - kernel instantiations with double population storage.
#include "engine_impl.cuh"

namespace pflbm {
Engine *make_engine_fp64(int q, bool jet, const HostParams &hp, uint32_t flags) {
    return make_engine_t<double>(q, jet, hp, flags);
}
}  // namespace pflbm
