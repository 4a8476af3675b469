// Serving loop: placeholder entry points (implemented in the next step).
#include "device.cuh"

using namespace elp;
extern "C" {
int elp_server_create(const elp_server_config*, elp_server** out) {
  if (out) *out = nullptr;
  set_error("server not available in this build");
  return ELP_ERR_STATE;
}
int elp_server_add_model(elp_server*, elp_model*, int*) { set_error("server not available"); return ELP_ERR_STATE; }
int elp_server_submit(elp_server*, int, const double*, int, double*, int64_t*) { set_error("server not available"); return ELP_ERR_STATE; }
int elp_server_wait(elp_server*, elp_request_result*, double) { set_error("server not available"); return ELP_ERR_STATE; }
int elp_server_destroy(elp_server*) { return ELP_OK; }
}
