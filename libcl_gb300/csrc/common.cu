// common.cu -- status strings, log sink, version, device helpers shared by the library.
#include <cstdio>
#include <mutex>

#include "internal.h"

namespace {
gbsph_log_fn g_log_fn = nullptr;
void* g_log_user = nullptr;
std::mutex g_log_mutex;
}  // namespace

namespace gbsph {

void log_msg(int level, const std::string& msg) {
    std::lock_guard<std::mutex> lock(g_log_mutex);
    if (g_log_fn) g_log_fn(level, msg.c_str(), g_log_user);
}

int fail(std::string* last_error, int status, const std::string& msg) {
    if (last_error) *last_error = msg;
    log_msg(0, msg);
    return status;
}

int dev_err_to_status(uint32_t bits) {
    if (bits == 0) return GBSPH_OK;
    if (bits & (DEV_ERR_LOOKBACK_TIMEOUT | DEV_ERR_MBAR_TIMEOUT | DEV_ERR_GRID_TIMEOUT)) return GBSPH_ERR_DEVICE_TIMEOUT;
    if (bits & DEV_ERR_KEY_RANGE) return GBSPH_ERR_DEVICE_RANGE;
    return GBSPH_ERR_STATE;
}

int num_sms() {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 148;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 148;
    return sms > 0 ? sms : 148;
}

}  // namespace gbsph

extern "C" {

GBSPH_API const char* gbsph_status_string(int status) {
    switch (status) {
        case GBSPH_OK: return "GBSPH_OK";
        case GBSPH_ERR_ARGUMENT: return "GBSPH_ERR_ARGUMENT";
        case GBSPH_ERR_SIZE_MISMATCH: return "GBSPH_ERR_SIZE_MISMATCH";
        case GBSPH_ERR_TOO_LARGE: return "GBSPH_ERR_TOO_LARGE";
        case GBSPH_ERR_BIT_RANGE: return "GBSPH_ERR_BIT_RANGE";
        case GBSPH_ERR_CUDA: return "GBSPH_ERR_CUDA";
        case GBSPH_ERR_DEVICE_TIMEOUT: return "GBSPH_ERR_DEVICE_TIMEOUT";
        case GBSPH_ERR_NOT_COMPILED: return "GBSPH_ERR_NOT_COMPILED";
        case GBSPH_ERR_OUT_OF_MEMORY: return "GBSPH_ERR_OUT_OF_MEMORY";
        case GBSPH_ERR_DEVICE_RANGE: return "GBSPH_ERR_DEVICE_RANGE";
        case GBSPH_ERR_STATE: return "GBSPH_ERR_STATE";
        default: return "GBSPH_ERR_UNKNOWN";
    }
}

GBSPH_API int gbsph_version(void) { return 1 * 10000 + 0 * 100 + 0; }

GBSPH_API void gbsph_set_logger(gbsph_log_fn fn, void* user) {
    std::lock_guard<std::mutex> lock(g_log_mutex);
    g_log_fn = fn;
    g_log_user = user;
}

}  // extern "C"
