/* wrl/client.h -- TEST INFRASTRUCTURE ONLY: empty stand-in (the reference's
 * CPU simulators hold no COM pointers). */
#pragma once
