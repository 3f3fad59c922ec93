// k_mac.cu — learned multipole-acceptance criterion (placeholder until the
// learned walk lands: every entry point reports GBH_ERR_UNSUPPORTED).
#include "gbh_ctx.h"

struct MacState {};

int enqueue_walk_learned(gbh_ctx* c) {
    c->last_error = "learned MAC walk not available";
    return GBH_ERR_UNSUPPORTED;
}

void mac_release(gbh_ctx* c) {
    delete c->mac;
    c->mac = nullptr;
}

extern "C" {
int gbh_mac_set_weights(gbh_ctx*, const float*, uint32_t) { return GBH_ERR_UNSUPPORTED; }
int gbh_mac_get_weights(gbh_ctx*, float*, uint32_t) { return GBH_ERR_UNSUPPORTED; }
int gbh_mac_generate(gbh_ctx*, const gbh_step_params*, uint32_t, uint64_t, uint32_t*) { return GBH_ERR_UNSUPPORTED; }
int gbh_mac_read_pairs(gbh_ctx*, float*, float*, uint32_t, uint32_t) { return GBH_ERR_UNSUPPORTED; }
int gbh_mac_write_pairs(gbh_ctx*, const float*, const float*, uint32_t) { return GBH_ERR_UNSUPPORTED; }
int gbh_mac_train(gbh_ctx*, uint32_t, uint32_t, float, uint64_t, float*) { return GBH_ERR_UNSUPPORTED; }
int gbh_mac_loss_grad(gbh_ctx*, const float*, const float*, uint32_t, float*, float*) { return GBH_ERR_UNSUPPORTED; }
int gbh_mac_predict(gbh_ctx*, const float*, uint32_t, float*) { return GBH_ERR_UNSUPPORTED; }
}
