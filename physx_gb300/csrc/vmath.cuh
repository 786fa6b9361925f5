// Device vector math for the GB300 rigid-body step.  Operation order follows
// PhysX's SSE2 vector layer (physx/include/foundation/PxVecMathSSE.h,
// PxVecQuat.h) and its scalar PxVec3/PxQuat types, so that contacts and solver
// rows reproduce the reference's rounding; the translation units that include
// this header are compiled with --fmad=false (no fused multiply-add).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <float.h>

namespace gbpx
{
struct V3 { float x, y, z; };
struct Q { float x, y, z, w; };
struct __align__(16) Tr { Q q; V3 p; };   // PxTransform fields (32 bytes in device arrays: whole sectors)
struct M33 { V3 c0, c1, c2; };     // column-major, as PxMat33 / Mat33V

__device__ __forceinline__ V3 v3(float x, float y, float z) { V3 r = {x, y, z}; return r; }
__device__ __forceinline__ V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 mul(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ V3 scale(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ V3 neg(V3 a) { return v3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ V3 vabs(V3 a) { return v3(fabsf(a.x), fabsf(a.y), fabsf(a.z)); }
__device__ __forceinline__ V3 vmin(V3 a, V3 b) { return v3(a.x < b.x ? a.x : b.x, a.y < b.y ? a.y : b.y, a.z < b.z ? a.z : b.z); }
__device__ __forceinline__ V3 vmax(V3 a, V3 b) { return v3(a.x > b.x ? a.x : b.x, a.y > b.y ? a.y : b.y, a.z > b.z ? a.z : b.z); }
// V3ScaleAdd(a, b, c) = a*b + c ; V3NegScaleSub(a, b, c) = c - a*b
__device__ __forceinline__ V3 scaleAdd(V3 a, float b, V3 c) { return add(scale(a, b), c); }
__device__ __forceinline__ V3 negScaleSub(V3 a, float b, V3 c) { return sub(c, scale(a, b)); }
// SSE2 V3Dot: (ay*by + aw*bw) + (ax*bx + az*bz) with w == 0
__device__ __forceinline__ float dotA(V3 a, V3 b) { return a.y * b.y + (a.x * b.x + a.z * b.z); }
// PxVec3::dot: (ax*bx + ay*by) + az*bz
__device__ __forceinline__ float dotS(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
__device__ __forceinline__ float sumElems(V3 a) { return (a.x + a.y) + a.z; }
__device__ __forceinline__ float lenSqA(V3 a) { return dotA(a, a); }
__device__ __forceinline__ float lenSqS(V3 a) { return dotS(a, a); }
// V3Normalize: a / sqrt(dot(a, a)) with an IEEE divide per lane
__device__ __forceinline__ V3 normalizeA(V3 a) { const float l = sqrtf(dotA(a, a)); return v3(a.x / l, a.y / l, a.z / l); }
__device__ __forceinline__ V3 scaleInv(V3 a, float b) { return v3(a.x / b, a.y / b, a.z / b); }
// PxVec3::getNormalized: a * (1 / |a|)
__device__ __forceinline__ V3 normalizeS(V3 a) { const float m = lenSqS(a); if(m > 0.0f) { const float r = 1.0f / sqrtf(m); return scale(a, r); } return v3(0, 0, 0); }
__device__ __forceinline__ V3 sel(bool c, V3 a, V3 b) { return c ? a : b; }
__device__ __forceinline__ float fsel(bool c, float a, float b) { return c ? a : b; }
__device__ __forceinline__ float fmin_(float a, float b) { return a < b ? a : b; }   // SSE minps: second operand on unordered
__device__ __forceinline__ float fmax_(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ float fclamp(float a, float lo, float hi) { return fmax_(fmin_(a, hi), lo); }
// V3RecipFast of the reference's SSE2 build (RCPPS): the reciprocal of the
// midpoint of the input's 2^-11 mantissa cell rounded to 13 significant bits
// (zero/denormal -> inf, inf -> 0, results below the normal range -> 0), which
// is what RCPPS returns on the x86 hosts that run the reference.
__device__ __forceinline__ float recipFast(float x)
{
	const uint32_t b = __float_as_uint(x);
	const uint32_t s = b & 0x80000000u, ex = (b >> 23) & 0xffu, i = (b >> 12) & 0x7ffu;
	uint32_t r;
	if(ex == 0xffu) r = (b & 0x7fffffu) ? (b | 0x400000u) : s;
	else if(ex == 0u) r = s | 0x7f800000u;
	else
	{
		const uint32_t D = 4097u + 2u * i;
		const uint32_t k = ((1u << 26) + D) / (2u * D);
		const int rex = 253 - int(ex);
		r = rex <= 0 ? s : (s | (uint32_t(rex) << 23) | ((k - 4096u) << 11));
	}
	return __uint_as_float(r);
}
// sin x and cos x of the integrator's half angles without double precision
// for |x| <= 0.125: each result is one rounding of a two-float value -- the
// leading Taylor terms (x - x^3/6, 1 - x^2/2) carried exactly by error-free
// transformations (the exact square and cube from FMA residuals, Dekker's
// fast two-sum) plus the rest of the Taylor series in single precision
// (truncated below 2^-54 relative).  The result is the correctly rounded
// sine / cosine unless that lies within about 2^-43 (relative) of a rounding
// boundary, the same values as evaluating in double and rounding.  Larger
// angles are evaluated in double.
__device__ __forceinline__ void sinCosAngle(float x, float& s, float& c)
{
	if(!(fabsf(x) <= 0.125f))
	{
		double ds, dc;
		sincos(double(x), &ds, &dc);
		s = float(ds);
		c = float(dc);
		return;
	}
	const float SIXTH_HI = 0.1666666716337204f, SIXTH_LO = -4.967053879312289e-09f;   // 1/6 = HI + LO to 2^-52
	const float x2 = x * x;
	const float x2e = fmaf(x, x, -x2);                  // x^2 = x2 + x2e exactly
	const float x3 = x2 * x;
	const float x3e = fmaf(x2, x, -x3) + x2e * x;       // x^3 = x3 + x3e
	const float t = x3 * SIXTH_HI;
	const float te = fmaf(x3, SIXTH_HI, -t) + (x3 * SIXTH_LO + x3e * SIXTH_HI);   // x^3/6 = t + te
	const float hs = x3 * x2 * (1.0f / 120.0f - x2 * (1.0f / 5040.0f - x2 * (1.0f / 362880.0f)));
	const float sh = x - t;
	const float se = (x - sh) - t;                      // x - t = sh + se exactly (|x| >= |t|)
	s = sh + ((se - te) + hs);
	const float a = 0.5f * x2, ae = 0.5f * x2e;         // x^2/2 = a + ae exactly
	const float hc = x2 * x2 * (1.0f / 24.0f - x2 * (1.0f / 720.0f - x2 * (1.0f / 40320.0f - x2 * (1.0f / 3628800.0f))));
	const float ch = 1.0f - a;
	const float ce = (1.0f - ch) - a;                   // 1 - a = ch + ce exactly
	c = ch + ((ce - ae) + hc);
}
__device__ __forceinline__ V3 unitX() { return v3(1, 0, 0); }
__device__ __forceinline__ V3 zero3() { return v3(0, 0, 0); }
__device__ __forceinline__ float getc(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

// ---- quaternions, aos order (PxVecQuat.h)
__device__ __forceinline__ V3 qv(Q q) { return v3(q.x, q.y, q.z); }
__device__ __forceinline__ V3 qRotate(Q q, V3 v)
{
	const float w2 = q.w * q.w + (-0.5f);
	const V3 a = scale(v, w2);
	const V3 u = qv(q);
	const V3 temp = scaleAdd(cross(u, v), q.w, a);
	return scale(scaleAdd(u, dotA(u, v), temp), 2.0f);
}
__device__ __forceinline__ V3 qRotateInv(Q q, V3 v)
{
	const float w2 = q.w * q.w + (-0.5f);
	const V3 a = scale(v, w2);
	const V3 u = qv(q);
	const V3 temp = negScaleSub(cross(u, v), q.w, a);
	return scale(scaleAdd(u, dotA(u, v), temp), 2.0f);
}
__device__ __forceinline__ V3 qBasis0(Q q)
{
	const float x2 = q.x * 2.0f, w2 = q.w * 2.0f;
	const V3 a = scale(qv(q), x2);
	const V3 ab = scaleAdd(v3(q.w, q.z, -q.y), w2, a);
	return v3(ab.x - 1.0f, ab.y, ab.z);
}
__device__ __forceinline__ V3 qBasis1(Q q)
{
	const float y2 = q.y * 2.0f, w2 = q.w * 2.0f;
	const V3 a = scale(qv(q), y2);
	const V3 ab = scaleAdd(v3(-q.z, q.w, q.x), w2, a);
	return v3(ab.x, ab.y - 1.0f, ab.z);
}
__device__ __forceinline__ V3 qBasis2(Q q)
{
	const float z2 = q.z * 2.0f, w2 = q.w * 2.0f;
	const V3 a = scale(qv(q), z2);
	const V3 ab = scaleAdd(v3(q.y, -q.x, q.w), w2, a);
	return v3(ab.x, ab.y, ab.z - 1.0f);
}
__device__ __forceinline__ Q qConj(Q q) { Q r = {-q.x, -q.y, -q.z, q.w}; return r; }
// QuatMul (aos): real = wa*wb - dot3(a, b) with V4Dot3 = (x + y) + z
__device__ __forceinline__ Q qMulA(Q a, Q b)
{
	const float d3 = (a.x * b.x + a.y * b.y) + a.z * b.z;
	const float real = a.w * b.w - d3;
	const V3 v0 = scale(qv(a), b.w), v1 = scale(qv(b), a.w), v2 = cross(qv(a), qv(b));
	const V3 im = add(add(v0, v1), v2);
	Q r = {im.x, im.y, im.z, real};
	return r;
}
// PxQuat::operator* (scalar)
__device__ __forceinline__ Q qMulS(Q a, Q b)
{
	Q r;
	r.x = a.w * b.x + b.w * a.x + a.y * b.z - b.y * a.z;
	r.y = a.w * b.y + b.w * a.y + a.z * b.x - b.z * a.x;
	r.z = a.w * b.z + b.w * a.z + a.x * b.y - b.x * a.y;
	r.w = a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z;
	return r;
}
// PxQuat::rotate / rotateInv (scalar)
__device__ __forceinline__ V3 qRotateS(Q q, V3 v)
{
	const float vx = 2.0f * v.x, vy = 2.0f * v.y, vz = 2.0f * v.z;
	const float w2 = q.w * q.w - 0.5f;
	const float dot2 = (q.x * vx + q.y * vy + q.z * vz);
	return v3((vx * w2 + (q.y * vz - q.z * vy) * q.w + q.x * dot2), (vy * w2 + (q.z * vx - q.x * vz) * q.w + q.y * dot2),
	          (vz * w2 + (q.x * vy - q.y * vx) * q.w + q.z * dot2));
}
__device__ __forceinline__ V3 qRotateInvS(Q q, V3 v)
{
	const float vx = 2.0f * v.x, vy = 2.0f * v.y, vz = 2.0f * v.z;
	const float w2 = q.w * q.w - 0.5f;
	const float dot2 = (q.x * vx + q.y * vy + q.z * vz);
	return v3((vx * w2 - (q.y * vz - q.z * vy) * q.w + q.x * dot2), (vy * w2 - (q.z * vx - q.x * vz) * q.w + q.y * dot2),
	          (vz * w2 - (q.x * vy - q.y * vx) * q.w + q.z * dot2));
}
__device__ __forceinline__ Q qNormalizeS(Q q)
{
	const float m = q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w;
	if(m != 0.0f) { const float s = 1.0f / sqrtf(m); Q r = {q.x * s, q.y * s, q.z * s, q.w * s}; return r; }
	return q;
}

// ---- transforms (aos PxTransformV)
__device__ __forceinline__ V3 trTransform(const Tr& t, V3 v) { return add(qRotate(t.q, v), t.p); }
__device__ __forceinline__ V3 trTransformInv(const Tr& t, V3 v) { return qRotateInv(t.q, sub(v, t.p)); }
// a.transformInv(b): (a^-1 * b)
__device__ __forceinline__ Tr trInvMul(const Tr& a, const Tr& b)
{
	Tr r;
	r.q = qMulA(qConj(a.q), b.q);
	r.p = qRotateInv(a.q, sub(b.p, a.p));
	return r;
}
// a.transform(b) = a * b
__device__ __forceinline__ Tr trMul(const Tr& a, const Tr& b)
{
	Tr r;
	r.q = qMulA(a.q, b.q);
	r.p = add(qRotate(a.q, b.p), a.p);
	return r;
}

// ---- 3x3 matrices
__device__ __forceinline__ V3 m33MulV(const M33& m, V3 v) { return add(add(scale(m.c0, v.x), scale(m.c1, v.y)), scale(m.c2, v.z)); }
__device__ __forceinline__ V3 m33TMulV(const M33& m, V3 v) { return v3(dotA(m.c0, v), dotA(m.c1, v), dotA(m.c2, v)); }
// PxMat33(q) scalar constructor
__device__ __forceinline__ M33 m33FromQuatS(Q q)
{
	const float x = q.x, y = q.y, z = q.z, w = q.w;
	const float x2 = x + x, y2 = y + y, z2 = z + z;
	const float xx = x2 * x, yy = y2 * y, zz = z2 * z;
	const float xy = x2 * y, xz = x2 * z, xw = x2 * w;
	const float yz = y2 * z, yw = y2 * w, zw = z2 * w;
	M33 m;
	m.c0 = v3(1.0f - yy - zz, xy + zw, xz - yw);
	m.c1 = v3(xy - zw, 1.0f - xx - zz, yz + xw);
	m.c2 = v3(xz + yw, yz - xw, 1.0f - xx - yy);
	return m;
}
// QuatGetMat33V, column-output SSE form (PxVecMathSSE.h:54), used by
// PxMatTransformV and PxMat33Padded: columns are v*2q_i + (2w*w - 1 / +-2w*q_j)
__device__ __forceinline__ M33 m33FromQuatCol(Q q)
{
	const float x2 = q.x + q.x, y2 = q.y + q.y, z2 = q.z + q.z, w2 = q.w + q.w;
	const float qx = x2 * q.w, qy = y2 * q.w, qz = z2 * q.w, qw = w2 * q.w + (-1.0f);
	M33 m;
	m.c0 = v3(q.x * x2 + qw, q.y * x2 + qz, q.z * x2 + (-qy));
	m.c1 = v3(q.x * y2 + (-qz), q.y * y2 + qw, q.z * y2 + qx);
	m.c2 = v3(q.x * z2 + qy, q.y * z2 + (-qx), q.z * z2 + qw);
	return m;
}
// PxMat33 * PxVec3 (scalar): c0*x + c1*y + c2*z
__device__ __forceinline__ V3 m33MulVS(const M33& m, V3 v)
{
	return v3(m.c0.x * v.x + m.c1.x * v.y + m.c2.x * v.z, m.c0.y * v.x + m.c1.y * v.y + m.c2.y * v.z,
	          m.c0.z * v.x + m.c1.z * v.y + m.c2.z * v.z);
}
} // namespace gbpx
