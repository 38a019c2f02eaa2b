// Project-written 4-vector (E, px, py, pz) with the operations the reference's 4-body code applies to
// MCBooster's Vector4R (include/goofit/PDFs/physics/detail/Dim5.h): v * w is the Minkowski product,
// dot / cross / d3mag act on the spatial parts (cross leaves the time component 0), mass2 = E^2 - |p|^2.
#pragma once
#include <cmath>
#include <mcbooster/GTypes.h>

namespace mcbooster {
class Vector4R {
    GReal_t v[4];

  public:
    Vector4R() : v{0, 0, 0, 0} {}
    Vector4R(GReal_t e, GReal_t px, GReal_t py, GReal_t pz) : v{e, px, py, pz} {}
    GReal_t get(int i) const { return v[i]; }
    void set(int i, GReal_t d) { v[i] = d; }
    void set(GReal_t e, GReal_t px, GReal_t py, GReal_t pz) {
        v[0] = e;
        v[1] = px;
        v[2] = py;
        v[3] = pz;
    }
    GReal_t mass2() const { return v[0] * v[0] - v[1] * v[1] - v[2] * v[2] - v[3] * v[3]; }
    GReal_t mass() const {
        const GReal_t m2 = mass2();
        return m2 > 0 ? std::sqrt(m2) : 0.0;
    }
    GReal_t d3mag() const { return std::sqrt(v[1] * v[1] + v[2] * v[2] + v[3] * v[3]); }
    GReal_t dot(const Vector4R &w) const { return v[1] * w.v[1] + v[2] * w.v[2] + v[3] * w.v[3]; }
    Vector4R cross(const Vector4R &w) const {
        return Vector4R(0.0, v[2] * w.v[3] - v[3] * w.v[2], v[3] * w.v[1] - v[1] * w.v[3], v[1] * w.v[2] - v[2] * w.v[1]);
    }
    Vector4R &operator+=(const Vector4R &w) {
        for(int i = 0; i < 4; ++i)
            v[i] += w.v[i];
        return *this;
    }
    Vector4R &operator-=(const Vector4R &w) {
        for(int i = 0; i < 4; ++i)
            v[i] -= w.v[i];
        return *this;
    }
    Vector4R &operator*=(GReal_t c) {
        for(int i = 0; i < 4; ++i)
            v[i] *= c;
        return *this;
    }
    Vector4R &operator/=(GReal_t c) {
        for(int i = 0; i < 4; ++i)
            v[i] /= c;
        return *this;
    }
    friend Vector4R operator+(Vector4R a, const Vector4R &b) { return a += b; }
    friend Vector4R operator-(Vector4R a, const Vector4R &b) { return a -= b; }
    friend Vector4R operator*(Vector4R a, GReal_t c) { return a *= c; }
    friend Vector4R operator*(GReal_t c, Vector4R a) { return a *= c; }
    friend Vector4R operator/(Vector4R a, GReal_t c) { return a /= c; }
    friend GReal_t operator*(const Vector4R &a, const Vector4R &b) {
        return a.v[0] * b.v[0] - a.v[1] * b.v[1] - a.v[2] * b.v[2] - a.v[3] * b.v[3];
    }
};
} // namespace mcbooster
