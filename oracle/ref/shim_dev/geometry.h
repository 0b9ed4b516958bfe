/* geometry.h stand-in for the device build of the reference's kernel sources
 * (oracle/ref/build_ref_dev.sh). The same vector/matrix types as the host stand-in
 * in ../shim/geometry.h (component-wise float arithmetic, operands by const
 * reference, results by value), with every function usable on host and device. */
#pragma once
#include <math.h>
#include <stdio.h>

#define HDFUNC __host__ __device__

__host__ __device__ inline float cmin(float a, float b) { return a < b ? a : b; }
__host__ __device__ inline float cmax(float a, float b) { return a > b ? a : b; }

struct cfloat2 {
    float x, y;
    __host__ __device__ cfloat2() {}
    __host__ __device__ cfloat2(float _x, float _y) : x(_x), y(_y) {}
    __host__ __device__ void Set(float _x, float _y) { x = _x; y = _y; }
};

struct cfloat3 {
    float x, y, z;
    __host__ __device__ cfloat3() {}
    __host__ __device__ cfloat3(float _x, float _y, float _z) : x(_x), y(_y), z(_z) {}
    __host__ __device__ void Set(float _x, float _y, float _z) { x = _x; y = _y; z = _z; }
    __host__ __device__ cfloat3 operator-(const cfloat3& b) const { return cfloat3(x - b.x, y - b.y, z - b.z); }
    __host__ __device__ cfloat3 operator+(const cfloat3& b) const { return cfloat3(x + b.x, y + b.y, z + b.z); }
    __host__ __device__ cfloat3 operator*(const cfloat3& b) const { return cfloat3(x * b.x, y * b.y, z * b.z); }
    __host__ __device__ cfloat3 operator/(const cfloat3& b) const { return cfloat3(x / b.x, y / b.y, z / b.z); }
    __host__ __device__ cfloat3 operator/(float b) const { return cfloat3(x / b, y / b, z / b); }
    __host__ __device__ cfloat3 operator*(float s) const { return cfloat3(x * s, y * s, z * s); }
    __host__ __device__ cfloat3 operator+(float a) const { return cfloat3(x + a, y + a, z + a); }
    __host__ __device__ cfloat3 operator-(float a) const { return cfloat3(x - a, y - a, z - a); }
    __host__ __device__ void operator+=(const cfloat3& b) { x += b.x; y += b.y; z += b.z; }
    __host__ __device__ void operator-=(const cfloat3& b) { x -= b.x; y -= b.y; z -= b.z; }
    __host__ __device__ void operator*=(float b) { x *= b; y *= b; z *= b; }
    __host__ __device__ void operator/=(float b) { x /= b; y /= b; z /= b; }
    __host__ __device__ void operator/=(const cfloat3& b) { x /= b.x; y /= b.y; z /= b.z; }
    __host__ __device__ float minx() const { return cmin(x, cmin(y, z)); }
};

__host__ __device__ inline cfloat3 minfilter(cfloat3 a, cfloat3 b) { return cfloat3(cmin(a.x, b.x), cmin(a.y, b.y), cmin(a.z, b.z)); }
__host__ __device__ inline cfloat3 maxfilter(cfloat3 a, cfloat3 b) { return cfloat3(cmax(a.x, b.x), cmax(a.y, b.y), cmax(a.z, b.z)); }
__host__ __device__ inline float dot(const cfloat3& a, const cfloat3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ inline cfloat3 cross(const cfloat3& a, const cfloat3& b) {
    return cfloat3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

struct cint3 {
    int x, y, z;
    __host__ __device__ cint3() {}
    __host__ __device__ cint3(int _x, int _y, int _z) : x(_x), y(_y), z(_z) {}
    __host__ __device__ void Set(int _x, int _y, int _z) { x = _x; y = _y; z = _z; }
    __host__ __device__ operator cfloat3() const { return cfloat3((float)x, (float)y, (float)z); }
    __host__ __device__ int prod() const { return x * y * z; }
    __host__ __device__ cint3 operator+(const cint3& b) const { return cint3(x + b.x, y + b.y, z + b.z); }
};

struct cmat3 {
    float data[9];
    __host__ __device__ cmat3() {}
    __host__ __device__ void Set(const float mat[]) { for (int i = 0; i < 9; i++) data[i] = mat[i]; }
    __host__ __device__ void Set(float c) { for (int i = 0; i < 9; i++) data[i] = c; }
    __host__ __device__ float* operator[](int i) { return &data[i * 3]; }
    __host__ __device__ const float* operator[](int i) const { return &data[i * 3]; }
    __host__ __device__ float Det() const {
        return data[0] * (data[4] * data[8] - data[5] * data[7]) + data[1] * (data[5] * data[6] - data[3] * data[8]) +
               data[2] * (data[3] * data[7] - data[4] * data[6]);
    }
};

__host__ __device__ inline void mat3add(const cmat3& a, const cmat3& b, cmat3& c) { for (int i = 0; i < 9; i++) c.data[i] = a.data[i] + b.data[i]; }
__host__ __device__ inline void mat3sub(const cmat3& a, const cmat3& b, cmat3& c) { for (int i = 0; i < 9; i++) c.data[i] = a.data[i] - b.data[i]; }
__host__ __device__ inline void mat3prod(const cmat3& a, const cmat3& b, cmat3& c) {
    cmat3 t;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            t.data[i * 3 + j] = a.data[i * 3] * b.data[j] + a.data[i * 3 + 1] * b.data[3 + j] + a.data[i * 3 + 2] * b.data[6 + j];
    c = t;
}
__host__ __device__ inline void mat3transpose(const cmat3& a, cmat3& b) {
    cmat3 t;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) t.data[i * 3 + j] = a.data[j * 3 + i];
    b = t;
}
__host__ __device__ inline void mvprod(const cmat3& m, const cfloat3& v, cfloat3& c) {
    cfloat3 t;
    t.x = m.data[0] * v.x + m.data[1] * v.y + m.data[2] * v.z;
    t.y = m.data[3] * v.x + m.data[4] * v.y + m.data[5] * v.z;
    t.z = m.data[6] * v.x + m.data[7] * v.y + m.data[8] * v.z;
    c = t;
}

struct cfloat4 {
    float x, y, z, w;
    __host__ __device__ void Set(float _x, float _y, float _z, float _w) { x = _x; y = _y; z = _z; w = _w; }
    __host__ __device__ cfloat4() : x(0), y(0), z(0), w(0) {}
    __host__ __device__ cfloat4(float _x, float _y, float _z, float _w) : x(_x), y(_y), z(_z), w(_w) {}
};
