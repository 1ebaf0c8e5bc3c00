/* Cube.hpp -- TEST INFRASTRUCTURE ONLY: the debug-cube type named by the
 * reference's Barnes-Hut sources (src/Render/Model/Cube.hpp); it draws nothing. */
#pragma once
#include <d3d11.h>
#include <SimpleMath.h>

class Cube {
public:
    explicit Cube(ID3D11DeviceContext*) {}
    void Render(DirectX::SimpleMath::Vector3, float, DirectX::SimpleMath::Matrix, bool = true) {}
};
