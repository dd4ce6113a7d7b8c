// Library-wide entry points of the C ABI (status strings, version).

#include "mt_common.cuh"

extern "C" {

const char* mt_status_string(int status) {
  switch (status) {
    case MT_OK:
      return "ok";
    case MT_ERR_INVALID_ARGUMENT:
      return "invalid argument";
    case MT_ERR_CUDA:
      return "CUDA launch error";
    case MT_ERR_WORKSPACE_TOO_SMALL:
      return "workspace too small";
    case MT_ERR_KEY_OVERFLOW:
      return "key field overflow";
    case MT_ERR_DEVICE_TIMEOUT:
      return "device spin-wait timed out";
    case MT_ERR_CAPACITY:
      return "output capacity exceeded";
    case MT_ERR_TOO_LARGE:
      return "size exceeds the static scratch limit";
    default:
      return "unknown status";
  }
}

int mt_version(void) { return (0 << 16) | 1; }

}  // extern "C"
