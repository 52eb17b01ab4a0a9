// Device vector algebra for the FP64 path.
//
// Every expression keeps the operand order of the reference expression it
// implements (Eigen expressions in pkg/dem/*.cpp), and the translation units
// that include this header are compiled with --fmad=false, so each result is the
// correctly rounded value of the same operation sequence a CPU evaluates.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace wg {

struct D3 {
    double x, y, z;
};
__host__ __device__ __forceinline__ D3 d3(double x, double y, double z) { return D3{x, y, z}; }
__host__ __device__ __forceinline__ D3 operator+(D3 a, D3 b) { return D3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__host__ __device__ __forceinline__ D3 operator-(D3 a, D3 b) { return D3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__host__ __device__ __forceinline__ D3 operator*(D3 a, double s) { return D3{a.x * s, a.y * s, a.z * s}; }
__host__ __device__ __forceinline__ D3 operator*(double s, D3 a) { return D3{s * a.x, s * a.y, s * a.z}; }
__host__ __device__ __forceinline__ D3 operator/(D3 a, double s) { return D3{a.x / s, a.y / s, a.z / s}; }
__host__ __device__ __forceinline__ double dot(D3 a, D3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__host__ __device__ __forceinline__ double sqn(D3 a) { return dot(a, a); }
__host__ __device__ __forceinline__ D3 cross(D3 a, D3 b) {
    return D3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__host__ __device__ __forceinline__ bool isZero(D3 a) { return a.x == 0 && a.y == 0 && a.z == 0; }
__host__ __device__ __forceinline__ double comp(D3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
__host__ __device__ __forceinline__ void setComp(D3& a, int i, double v) {
    if (i == 0) a.x = v; else if (i == 1) a.y = v; else a.z = v;
}
// Eigen's normalize(): divide by sqrt(squaredNorm) when positive
__host__ __device__ __forceinline__ D3 normalized(D3 a) {
    double z = sqn(a);
    return z > 0 ? a / sqrt(z) : a;
}
// std::min / std::max semantics (first argument wins ties)
__host__ __device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }
__host__ __device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }

struct DQ {
    double w, x, y, z;
};
__host__ __device__ __forceinline__ DQ qmul(DQ a, DQ b) {
    DQ r;
    r.w = ((a.w * b.w - a.x * b.x) - a.y * b.y) - a.z * b.z;
    r.x = ((a.w * b.x + a.x * b.w) + a.y * b.z) - a.z * b.y;
    r.y = ((a.w * b.y + a.y * b.w) + a.z * b.x) - a.x * b.z;
    r.z = ((a.w * b.z + a.z * b.w) + a.x * b.y) - a.y * b.x;
    return r;
}
__host__ __device__ __forceinline__ DQ qnormalized(DQ q) {
    double n = sqrt(((q.x * q.x + q.y * q.y) + q.z * q.z) + q.w * q.w);
    return DQ{q.w / n, q.x / n, q.y / n, q.z / n};
}
// Rotation matrix (given by its three columns) to quaternion, Shepperd's method:
// trace branch when positive, else the largest diagonal element picks the branch.
__host__ __device__ __forceinline__ DQ quatFromCols(D3 c0, D3 c1, D3 c2) {
    // m[r][c] = column c, row r
    double m[3][3] = {{c0.x, c1.x, c2.x}, {c0.y, c1.y, c2.y}, {c0.z, c1.z, c2.z}};
    DQ q;
    double t = (m[0][0] + m[1][1]) + m[2][2];
    if (t > 0) {
        t = sqrt(t + 1.0);
        q.w = 0.5 * t;
        t = 0.5 / t;
        q.x = (m[2][1] - m[1][2]) * t;
        q.y = (m[0][2] - m[2][0]) * t;
        q.z = (m[1][0] - m[0][1]) * t;
    } else {
        int i = 0;
        if (m[1][1] > m[0][0]) i = 1;
        if (m[2][2] > m[i][i]) i = 2;
        int j = (i + 1) % 3, k = (j + 1) % 3;
        t = sqrt(((m[i][i] - m[j][j]) - m[k][k]) + 1.0);
        double c[3];
        c[i] = 0.5 * t;
        t = 0.5 / t;
        q.w = (m[k][j] - m[j][k]) * t;
        c[j] = (m[j][i] + m[i][j]) * t;
        c[k] = (m[k][i] + m[i][k]) * t;
        q.x = c[0];
        q.y = c[1];
        q.z = c[2];
    }
    return q;
}
// v' = v + w*(2 q x v) + q x (2 q x v)
__host__ __device__ __forceinline__ D3 qrot(DQ q, D3 v) {
    D3 qv{q.x, q.y, q.z};
    D3 uv = cross(qv, v);
    uv = uv + uv;
    return (v + q.w * uv) + cross(qv, uv);
}

// 3x3 matrix stored row-major
struct DM3 {
    double m[9];
};
__host__ __device__ __forceinline__ D3 mul(const DM3& A, D3 v) {
    return D3{(A.m[0] * v.x + A.m[1] * v.y) + A.m[2] * v.z, (A.m[3] * v.x + A.m[4] * v.y) + A.m[5] * v.z,
              (A.m[6] * v.x + A.m[7] * v.y) + A.m[8] * v.z};
}

}  // namespace wg
