// Double-single arithmetic shared by the ILU(0) sweeps and the Krylov basis.
//
// A value held as the unevaluated sum hi + lo of two floats (|lo| at most
// half an ulp of hi): 48 significand bits on the FP32 pipes, which on this
// part issue 64 times as many operations per clock as the FP64 pipe.  The
// arithmetic is built from the error-free transformations of Knuth's two-sum
// (a + b = s + e exactly) and of the fused-multiply-add two-product
// (a * b = p + e exactly, e = fma(a, b, -p)); a product's cross terms and the
// final addition of the low parts are rounded once each (the "sloppy"
// double-single sum), so an operation errs by a few units of 2^-48 of its
// operands: not bit-identical to FP64, within a few 2^-48 of it.
#pragma once
#include <cuda_runtime.h>

struct __align__(8) dsf { float hi, lo; };

__device__ __forceinline__ dsf ds_two_sum(float a, float b)
{
	const float s = a + b, v = s - a;
	return dsf{ s, (a - (s - v)) + (b - v) };
}

__device__ __forceinline__ dsf ds_fast_two_sum(float a, float b)     // |a| >= |b|
{
	const float s = a + b;
	return dsf{ s, b - (s - a) };
}

// c + a * b
__device__ __forceinline__ dsf ds_fma(dsf a, dsf b, dsf c)
{
	const float p = a.hi * b.hi;
	float e = fmaf(a.hi, b.hi, -p);
	e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
	dsf s = ds_two_sum(c.hi, p);
	s.lo += e + c.lo;
	return ds_fast_two_sum(s.hi, s.lo);
}

__host__ __device__ __forceinline__ dsf ds_neg(dsf a) { return dsf{ -a.hi, -a.lo }; }

__device__ __forceinline__ dsf ds_from(double v)
{
	const float h = __double2float_rn(v);
	return dsf{ h, __double2float_rn(v - (double)h) };
}


__device__ __forceinline__ double ds_to_double(dsf a) { return (double)a.hi + (double)a.lo; }
