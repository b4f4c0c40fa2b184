// nbody::Vector for this library's host layer: three floats with the arithmetic the
// solver interface and its callers use (the reference's include/nbody/vector.h exposes the
// same type, layout and operators; a build inside the reference uses that header instead).
#pragma once
#include <cmath>
#include <cstddef>

namespace nbody
{
    struct Vector
    {
        float x = 0;
        float y = 0;
        float z = 0;

        float& operator[](std::size_t i) { return i == 0 ? x : (i == 1 ? y : z); }
        const float& operator[](std::size_t i) const { return i == 0 ? x : (i == 1 ? y : z); }

        bool operator==(const Vector& o) const = default;
        Vector operator+(const Vector& o) const { return { x + o.x, y + o.y, z + o.z }; }
        Vector operator-(const Vector& o) const { return { x - o.x, y - o.y, z - o.z }; }
        Vector operator*(const float s) const { return { x * s, y * s, z * s }; }
        Vector operator/(const float s) const { return { x / s, y / s, z / s }; }
        Vector& operator+=(const Vector& o) { x += o.x; y += o.y; z += o.z; return *this; }
        Vector& operator-=(const Vector& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }

        [[nodiscard]] float size_sq() const { return x * x + y * y + z * z; }
        [[nodiscard]] float size() const { return std::sqrt(size_sq()); }
        [[nodiscard]] float dist_sq(const Vector& o) const { return (o - *this).size_sq(); }
    };

    inline Vector operator*(const float s, const Vector& v) { return v * s; }
    inline float dot(const Vector& a, const Vector& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
}
