// Continuous-batching server and autotuner (filled in below the core engine).
#include "../../include/sop_gpu.h"

extern "C" int sop_autotune(sop_engine*, int, char*, int) { return SOP_ERR_UNSUPPORTED; }
extern "C" int sop_server_create(const sop_server_config*, sop_server**) { return SOP_ERR_UNSUPPORTED; }
extern "C" int sop_server_destroy(sop_server*) { return SOP_ERR_UNSUPPORTED; }
extern "C" int sop_server_submit(sop_server*, const sop_system_desc*, int64_t, int64_t*) {
  return SOP_ERR_UNSUPPORTED;
}
extern "C" int sop_server_pump(sop_server*, int*) { return SOP_ERR_UNSUPPORTED; }
extern "C" int sop_server_poll(sop_server*, sop_request_result*, int, int*) { return SOP_ERR_UNSUPPORTED; }
extern "C" int sop_server_clock(sop_server*, double*) { return SOP_ERR_UNSUPPORTED; }
extern "C" int sop_server_stats(sop_server*, int64_t*, int*, int*) { return SOP_ERR_UNSUPPORTED; }
