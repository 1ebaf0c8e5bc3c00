/* GeometricPrimitive.h -- TEST INFRASTRUCTURE ONLY: the DirectXTK primitive
 * type named by the reference's Barnes-Hut sources; it draws nothing. */
#pragma once
#include <memory>
#include "d3d11.h"

namespace DirectX {
class GeometricPrimitive {
public:
    static std::unique_ptr<GeometricPrimitive> CreateSphere(ID3D11DeviceContext*) { return nullptr; }
};
}  // namespace DirectX
