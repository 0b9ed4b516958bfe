/* geometry.h stand-in for the oracle host build (oracle/ref).
 *
 * The reference's SPH_Solver/catpaw/geometry.h binds temporaries to non-const
 * references (e.g. `cfloat3 operator-(cfloat3& b)` applied to an rvalue), which
 * only MSVC accepts, and returns a reference to a temporary from
 * `operator/(float)`. This header gives the same vector/matrix types with the
 * same component-wise float arithmetic, taking operands by const reference
 * and returning by value, so the reference kernel sources compile with g++. */
#pragma once
#include <math.h>
#include <stdio.h>
#include "cudashim.h"

#define HDFUNC

inline float cmin(float a, float b) { return a < b ? a : b; }
inline float cmax(float a, float b) { return a > b ? a : b; }

struct cfloat2 {
    float x, y;
    cfloat2() {}
    cfloat2(float _x, float _y) : x(_x), y(_y) {}
    void Set(float _x, float _y) { x = _x; y = _y; }
};

struct cfloat3 {
    float x, y, z;
    cfloat3() {}
    cfloat3(float _x, float _y, float _z) : x(_x), y(_y), z(_z) {}
    void Set(float _x, float _y, float _z) { x = _x; y = _y; z = _z; }
    cfloat3 operator-(const cfloat3& b) const { return cfloat3(x - b.x, y - b.y, z - b.z); }
    cfloat3 operator+(const cfloat3& b) const { return cfloat3(x + b.x, y + b.y, z + b.z); }
    cfloat3 operator*(const cfloat3& b) const { return cfloat3(x * b.x, y * b.y, z * b.z); }
    cfloat3 operator/(const cfloat3& b) const { return cfloat3(x / b.x, y / b.y, z / b.z); }
    cfloat3 operator/(float b) const { return cfloat3(x / b, y / b, z / b); }
    cfloat3 operator*(float s) const { return cfloat3(x * s, y * s, z * s); }
    cfloat3 operator+(float a) const { return cfloat3(x + a, y + a, z + a); }
    cfloat3 operator-(float a) const { return cfloat3(x - a, y - a, z - a); }
    void operator+=(const cfloat3& b) { x += b.x; y += b.y; z += b.z; }
    void operator-=(const cfloat3& b) { x -= b.x; y -= b.y; z -= b.z; }
    void operator*=(float b) { x *= b; y *= b; z *= b; }
    void operator/=(float b) { x /= b; y /= b; z /= b; }
    void operator/=(const cfloat3& b) { x /= b.x; y /= b.y; z /= b.z; }
    float minx() const { return cmin(x, cmin(y, z)); }
};

inline cfloat3 minfilter(cfloat3 a, cfloat3 b) { return cfloat3(cmin(a.x, b.x), cmin(a.y, b.y), cmin(a.z, b.z)); }
inline cfloat3 maxfilter(cfloat3 a, cfloat3 b) { return cfloat3(cmax(a.x, b.x), cmax(a.y, b.y), cmax(a.z, b.z)); }
inline float dot(const cfloat3& a, const cfloat3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline cfloat3 cross(const cfloat3& a, const cfloat3& b) {
    return cfloat3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

struct cint3 {
    int x, y, z;
    cint3() {}
    cint3(int _x, int _y, int _z) : x(_x), y(_y), z(_z) {}
    void Set(int _x, int _y, int _z) { x = _x; y = _y; z = _z; }
    operator cfloat3() const { return cfloat3((float)x, (float)y, (float)z); }
    int prod() const { return x * y * z; }
    cint3 operator+(const cint3& b) const { return cint3(x + b.x, y + b.y, z + b.z); }
};

struct cmat3 {
    float data[9];
    cmat3() {}
    void Set(const float mat[]) { for (int i = 0; i < 9; i++) data[i] = mat[i]; }
    void Set(float c) { for (int i = 0; i < 9; i++) data[i] = c; }
    float* operator[](int i) { return &data[i * 3]; }
    const float* operator[](int i) const { return &data[i * 3]; }
    float Det() const {
        return data[0] * (data[4] * data[8] - data[5] * data[7]) + data[1] * (data[5] * data[6] - data[3] * data[8]) +
               data[2] * (data[3] * data[7] - data[4] * data[6]);
    }
};

inline void mat3add(const cmat3& a, const cmat3& b, cmat3& c) { for (int i = 0; i < 9; i++) c.data[i] = a.data[i] + b.data[i]; }
inline void mat3sub(const cmat3& a, const cmat3& b, cmat3& c) { for (int i = 0; i < 9; i++) c.data[i] = a.data[i] - b.data[i]; }
inline void mat3prod(const cmat3& a, const cmat3& b, cmat3& c) {
    cmat3 t;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            t.data[i * 3 + j] = a.data[i * 3] * b.data[j] + a.data[i * 3 + 1] * b.data[3 + j] + a.data[i * 3 + 2] * b.data[6 + j];
    c = t;
}
inline void mat3transpose(const cmat3& a, cmat3& b) {
    cmat3 t;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) t.data[i * 3 + j] = a.data[j * 3 + i];
    b = t;
}
inline void mvprod(const cmat3& m, const cfloat3& v, cfloat3& c) {
    cfloat3 t;
    t.x = m.data[0] * v.x + m.data[1] * v.y + m.data[2] * v.z;
    t.y = m.data[3] * v.x + m.data[4] * v.y + m.data[5] * v.z;
    t.z = m.data[6] * v.x + m.data[7] * v.y + m.data[8] * v.z;
    c = t;
}

struct cfloat4 {
    float x, y, z, w;
    void Set(float _x, float _y, float _z, float _w) { x = _x; y = _y; z = _z; w = _w; }
    cfloat4() : x(0), y(0), z(0), w(0) {}
    cfloat4(float _x, float _y, float _z, float _w) : x(_x), y(_y), z(_z), w(_w) {}
};
