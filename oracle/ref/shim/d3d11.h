/* d3d11.h -- TEST INFRASTRUCTURE ONLY: opaque Direct3D 11 type names, so that
 * the reference's CPU N-body sources compile with g++.  Nothing is defined:
 * the reference's CPU simulators are created with a null device context. */
#pragma once
struct ID3D11Device;
struct ID3D11DeviceContext;
struct ID3D11Buffer;
