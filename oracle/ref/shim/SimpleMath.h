/*
 * SimpleMath.h -- TEST INFRASTRUCTURE ONLY: a type-only stand-in for the
 * DirectXTK SimpleMath header, so that the reference's CPU N-body sources
 * (src/Sim/Octree.cpp, BarnesHut.cpp, BruteForceCPU.cpp, Physics.hpp) compile
 * unmodified with g++ for the oracle's parity check.
 *
 * DirectXTK is an un-vendored submodule of the reference (lib/DirectXTK is
 * empty; its pinned commit is not recoverable), so this header is written from
 * the library's documented interface, not from its source.  It declares only
 * what those files use.  The arithmetic is the documented meaning of each
 * operation in plain float, evaluated in the order written here:
 *   Vector3 +, -, * float, componentwise;   Vector3 /= s  ->  v * (1.f / s);
 *   Length() = sqrtf((x*x + y*y) + z*z);    Normalize(): v / Length(), zero
 *   stays zero;  DistanceSquared(a, b) = the same dot of (b - a).
 * This arithmetic is the part of the reference build that stays unpinned
 * (DirectXMath's SIMD code may round differently by an ulp); the recursion,
 * ordering and branch logic of the reference files are their own.
 * Matrix and Color carry data only; nothing here renders.
 */
#pragma once
#include <cmath>

namespace DirectX {
namespace SimpleMath {

struct Vector3 {
    float x, y, z;
    Vector3() : x(0.f), y(0.f), z(0.f) {}
    Vector3(float ax, float ay, float az) : x(ax), y(ay), z(az) {}

    float LengthSquared() const { return (x * x + y * y) + z * z; }
    float Length() const { return std::sqrt(LengthSquared()); }
    void Normalize() {
        const float len = Length();
        if (len > 0.f) { x = x / len; y = y / len; z = z / len; }
        else { x = y = z = 0.f; }
    }
    Vector3& operator+=(const Vector3& v) { x = x + v.x; y = y + v.y; z = z + v.z; return *this; }
    Vector3& operator-=(const Vector3& v) { x = x - v.x; y = y - v.y; z = z - v.z; return *this; }
    Vector3& operator*=(float s) { x = x * s; y = y * s; z = z * s; return *this; }
    Vector3& operator/=(float s) { const float r = 1.f / s; return *this *= r; }

    static float DistanceSquared(const Vector3& a, const Vector3& b) {
        const Vector3 d(b.x - a.x, b.y - a.y, b.z - a.z);
        return d.LengthSquared();
    }
};
inline Vector3 operator+(const Vector3& a, const Vector3& b) { return Vector3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline Vector3 operator-(const Vector3& a, const Vector3& b) { return Vector3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline Vector3 operator*(const Vector3& a, float s) { return Vector3(a.x * s, a.y * s, a.z * s); }
inline Vector3 operator/(const Vector3& a, float s) { const float r = 1.f / s; return a * r; }

struct Color {
    float r, g, b, a;
    Color() : r(0.f), g(0.f), b(0.f), a(1.f) {}
    Color(float ar, float ag, float ab) : r(ar), g(ag), b(ab), a(1.f) {}
    Color(float ar, float ag, float ab, float aa) : r(ar), g(ag), b(ab), a(aa) {}
};

struct Matrix {
    float m[4][4];
    Matrix() : m{{1.f, 0.f, 0.f, 0.f}, {0.f, 1.f, 0.f, 0.f}, {0.f, 0.f, 1.f, 0.f}, {0.f, 0.f, 0.f, 1.f}} {}
    static Matrix CreateScale(float s) {
        Matrix r;
        r.m[0][0] = r.m[1][1] = r.m[2][2] = s;
        return r;
    }
    static Matrix CreateTranslation(const Vector3& t) {
        Matrix r;
        r.m[3][0] = t.x; r.m[3][1] = t.y; r.m[3][2] = t.z;
        return r;
    }
};
inline Matrix operator*(const Matrix& a, const Matrix& b) {
    Matrix r;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            float s = 0.f;
            for (int k = 0; k < 4; ++k) s += a.m[i][k] * b.m[k][j];
            r.m[i][j] = s;
        }
    return r;
}

}  // namespace SimpleMath
}  // namespace DirectX
