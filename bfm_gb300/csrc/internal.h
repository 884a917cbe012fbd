/* Library-internal helpers shared by the translation units (not exported). */
#pragma once

#ifdef __cplusplus
extern "C" {
#endif

/* Set the message bfm_gpu_last_error() reports on this thread. */
__attribute__((visibility("hidden"))) void bfm_gpu_set_last_error(const char* msg);

#ifdef __cplusplus
}
#endif
