/* Log.hpp -- TEST INFRASTRUCTURE ONLY: the reference's logging macros as
 * no-ops (src/Services/Log.hpp writes to the UI log). */
#pragma once
#define LOGV(str)
#define LOGM(str)
#define LOGW(str)
#define LOGE(str)
