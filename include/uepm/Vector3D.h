// Vector3D.h -- the reference's small 3-vector value type (src/EPP/Vector3D.h, Vector3D.inl),
// re-provided with the same interface (members X, Y, Z; '*' is the dot product, '%' the cross
// product) so that code written against src/EPP compiles unchanged.
#pragma once

#include <cmath>
#include <iostream>
#include <tuple>

template <typename T>
class Vector3D {
 public:
    T X;
    T Y;
    T Z;

    Vector3D() : X(0), Y(0), Z(0) {}
    Vector3D(const T& v) : X(v), Y(v), Z(v) {}
    template <typename O>
    Vector3D(const Vector3D<O>& o) : X(o.X), Y(o.Y), Z(o.Z) {}
    explicit Vector3D(const T& x, const T& y, const T& z) : X(x), Y(y), Z(z) {}

    template <typename O>
    Vector3D& operator=(const Vector3D<O>& o) {
        X = o.X;
        Y = o.Y;
        Z = o.Z;
        return *this;
    }

    const Vector3D& operator+() const { return *this; }
    Vector3D        operator-() const { return Vector3D(-X, -Y, -Z); }

    template <typename O>
    Vector3D operator+(const Vector3D<O>& o) const {
        return Vector3D(X + o.X, Y + o.Y, Z + o.Z);
    }
    template <typename O>
    Vector3D operator-(const Vector3D<O>& o) const {
        return Vector3D(X - o.X, Y - o.Y, Z - o.Z);
    }
    // dot product
    template <typename O>
    T operator*(const Vector3D<O>& o) const {
        return X * o.X + Y * o.Y + Z * o.Z;
    }
    // cross product
    template <typename O>
    Vector3D operator%(const Vector3D<O>& o) const {
        return Vector3D(Y * o.Z - Z * o.Y, Z * o.X - X * o.Z, X * o.Y - Y * o.X);
    }
    Vector3D operator*(T s) const { return Vector3D(X * s, Y * s, Z * s); }
    Vector3D operator/(T s) const { return Vector3D(X / s, Y / s, Z / s); }

    template <typename O>
    Vector3D& operator+=(const Vector3D<O>& o) {
        return *this = *this + o;
    }
    template <typename O>
    Vector3D& operator-=(const Vector3D<O>& o) {
        return *this = *this - o;
    }
    template <typename O>
    Vector3D& operator%=(const Vector3D<O>& o) {
        return *this = *this % o;
    }
    Vector3D& operator*=(T s) { return *this = *this * s; }
    Vector3D& operator/=(T s) { return *this = *this / s; }

    double Length() const {
        const double w = *this * *this;
        return std::sqrt(w);
    }
    Vector3D Normalize() const {
        const T len = Length();
        return (len != 0) ? *this / len : *this;
    }

    // Rodrigues rotation of this vector about `axis` by `angle` (radians).
    template <typename O, typename A>
    Vector3D RotateAround(const Vector3D<O>& axis, A angle) const {
        const Vector3D<O> u  = axis.Normalize();
        const T           c  = std::cos(angle), s = std::sin(angle), om = T(1) - c;
        Vector3D          r;
        r.X = (c + om * u.X * u.X) * X + (om * u.X * u.Y - u.Z * s) * Y + (om * u.X * u.Z + u.Y * s) * Z;
        r.Y = (om * u.X * u.Y + u.Z * s) * X + (c + om * u.Y * u.Y) * Y + (om * u.Y * u.Z - u.X * s) * Z;
        r.Z = (om * u.X * u.Z - u.Y * s) * X + (om * u.Y * u.Z + u.X * s) * Y + (c + om * u.Z * u.Z) * Z;
        return r;
    }
    template <typename O, typename A>
    Vector3D RotateTowards(const Vector3D<O>& other, A angle) const {
        return RotateAround(*this % other, angle);
    }

    double getTheta() const {
        double ct = Z / Length();
        if (std::isnan(ct) || std::isinf(ct) || ct > 1. || ct < -1) ct = (ct < 0 ? -1 : 1);
        return std::acos(ct);
    }
    double getPhi() const { return std::atan2(Y, X); }

    // cosine of the angle between two vectors; 1 when either is (numerically) zero
    friend double compute_cos_angle(const Vector3D& a, const Vector3D& b) {
        const double dp = a * b;
        const double np = a.Length() * b.Length();
        return (np < 1.0e-13) ? 1.0 : dp / (a.Length() * b.Length());
    }

    friend std::ostream& operator<<(std::ostream& os, const Vector3D& v) {
        return os << "(" << v.X << ", " << v.Y << ", " << v.Z << ")";
    }
};

template <typename T>
Vector3D<T> operator*(T s, const Vector3D<T>& v) {
    return v * s;
}
template <typename T>
Vector3D<T> operator/(T s, const Vector3D<T>& v) {
    return v / s;
}
template <typename T>
Vector3D<T> cross_product(const Vector3D<T>& a, const Vector3D<T>& b) {
    return a % b;
}
template <typename T>
bool operator==(const Vector3D<T>& a, const Vector3D<T>& b) {
    return a.X == b.X && a.Y == b.Y && a.Z == b.Z;
}
template <typename T>
bool operator<(const Vector3D<T>& a, const Vector3D<T>& b) {
    return std::tie(a.X, a.Y, a.Z) < std::tie(b.X, b.Y, b.Z);
}
