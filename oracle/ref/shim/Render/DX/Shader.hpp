/* Shader.hpp -- TEST INFRASTRUCTURE ONLY: empty stand-in (included by
 * src/Sim/BruteForceCPU.cpp, which uses nothing from it). */
#pragma once
