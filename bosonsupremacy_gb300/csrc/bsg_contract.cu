// Transfer contraction: placeholder until the tcgen05 kernel lands.
#include "bsg_internal.h"
extern "C" int bsg_pattern_amplitudes(bsg_handle_t, const void* const*, const double*, int, int, int, const int32_t*,
                                      int64_t, int, double*, bsg_stream_t) {
  bsg::set_error("bsg_pattern_amplitudes: not built yet");
  return BSG_ERR_LIMIT;
}
