/* ConstantBuffer.hpp -- TEST INFRASTRUCTURE ONLY: empty stand-in (included by
 * src/Sim/BruteForceCPU.hpp, which uses nothing from it). */
#pragma once
