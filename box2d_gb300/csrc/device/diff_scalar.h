/*
 * Scalars for differentiating the step along a recorded trajectory.
 *
 * b2dDual<T, N> carries a float primal and N tangents of type T. Every primal operation
 * is the plain float operation in the order the expression is written, so with contraction
 * off (nvcc --fmad=false, gcc -ffp-contract=off) the primal of a dual computation equals
 * the forward step's float result bit for bit, and every branch the forward took is taken
 * again. Tangents follow the chain rule in T (float on the device, double on the host).
 */
#pragma once

#include <math.h>

#ifdef __CUDACC__
#define B2D_HD __host__ __device__ __forceinline__
#define B2D_HDM __host__ __device__ __forceinline__
#else
#define B2D_HD static inline
#define B2D_HDM inline
#endif

template <class T, int N> struct b2dDual
{
	float v;
	T d[N];
	/* a constant: zero tangents */
	static B2D_HDM b2dDual make( float x )
	{
		b2dDual r;
		r.v = x;
		for ( int i = 0; i < N; ++i ) r.d[i] = T( 0 );
		return r;
	}
};

template <class T, int N> B2D_HD b2dDual<T, N> operator+( const b2dDual<T, N>& a, const b2dDual<T, N>& b )
{
	b2dDual<T, N> r;
	r.v = a.v + b.v;
	for ( int i = 0; i < N; ++i ) r.d[i] = a.d[i] + b.d[i];
	return r;
}

template <class T, int N> B2D_HD b2dDual<T, N> operator-( const b2dDual<T, N>& a, const b2dDual<T, N>& b )
{
	b2dDual<T, N> r;
	r.v = a.v - b.v;
	for ( int i = 0; i < N; ++i ) r.d[i] = a.d[i] - b.d[i];
	return r;
}

template <class T, int N> B2D_HD b2dDual<T, N> operator-( const b2dDual<T, N>& a )
{
	b2dDual<T, N> r;
	r.v = -a.v;
	for ( int i = 0; i < N; ++i ) r.d[i] = -a.d[i];
	return r;
}

template <class T, int N> B2D_HD b2dDual<T, N> operator*( const b2dDual<T, N>& a, const b2dDual<T, N>& b )
{
	b2dDual<T, N> r;
	r.v = a.v * b.v;
	for ( int i = 0; i < N; ++i ) r.d[i] = a.d[i] * T( b.v ) + T( a.v ) * b.d[i];
	return r;
}

template <class T, int N> B2D_HD b2dDual<T, N> operator/( const b2dDual<T, N>& a, const b2dDual<T, N>& b )
{
	b2dDual<T, N> r;
	r.v = a.v / b.v;
	for ( int i = 0; i < N; ++i ) r.d[i] = ( a.d[i] - T( r.v ) * b.d[i] ) / T( b.v );
	return r;
}

/* mixed operations with float constants */
template <class T, int N> B2D_HD b2dDual<T, N> operator+( const b2dDual<T, N>& a, float b )
{
	b2dDual<T, N> r = a;
	r.v = a.v + b;
	return r;
}
template <class T, int N> B2D_HD b2dDual<T, N> operator+( float a, const b2dDual<T, N>& b )
{
	b2dDual<T, N> r = b;
	r.v = a + b.v;
	return r;
}
template <class T, int N> B2D_HD b2dDual<T, N> operator-( const b2dDual<T, N>& a, float b )
{
	b2dDual<T, N> r = a;
	r.v = a.v - b;
	return r;
}
template <class T, int N> B2D_HD b2dDual<T, N> operator-( float a, const b2dDual<T, N>& b )
{
	b2dDual<T, N> r;
	r.v = a - b.v;
	for ( int i = 0; i < N; ++i ) r.d[i] = -b.d[i];
	return r;
}
template <class T, int N> B2D_HD b2dDual<T, N> operator*( const b2dDual<T, N>& a, float b )
{
	b2dDual<T, N> r;
	r.v = a.v * b;
	for ( int i = 0; i < N; ++i ) r.d[i] = a.d[i] * T( b );
	return r;
}
template <class T, int N> B2D_HD b2dDual<T, N> operator*( float a, const b2dDual<T, N>& b )
{
	b2dDual<T, N> r;
	r.v = a * b.v;
	for ( int i = 0; i < N; ++i ) r.d[i] = T( a ) * b.d[i];
	return r;
}
template <class T, int N> B2D_HD b2dDual<T, N> operator/( float a, const b2dDual<T, N>& b )
{
	b2dDual<T, N> r;
	r.v = a / b.v;
	for ( int i = 0; i < N; ++i ) r.d[i] = -T( r.v ) * b.d[i] / T( b.v );
	return r;
}

template <class T, int N> B2D_HD b2dDual<T, N> b2dSqrt( const b2dDual<T, N>& a )
{
	b2dDual<T, N> r;
	r.v = sqrtf( a.v );
	for ( int i = 0; i < N; ++i ) r.d[i] = r.v > 0.0f ? a.d[i] / ( T( 2 ) * T( r.v ) ) : T( 0 );
	return r;
}

/* select keeps the chosen operand's tangents: the derivative of the branch taken */
template <class T, int N> B2D_HD b2dDual<T, N> b2dMin( const b2dDual<T, N>& a, const b2dDual<T, N>& b ) { return a.v < b.v ? a : b; }
template <class T, int N> B2D_HD b2dDual<T, N> b2dMax( const b2dDual<T, N>& a, const b2dDual<T, N>& b ) { return a.v > b.v ? a : b; }
template <class T, int N> B2D_HD b2dDual<T, N> b2dClamp( const b2dDual<T, N>& a, float lo, float hi )
{
	return a.v < lo ? b2dDual<T, N>::make( lo ) : ( a.v > hi ? b2dDual<T, N>::make( hi ) : a );
}

/* 2-vectors and rotations over a dual scalar */
template <class S> struct b2dVec2
{
	S x, y;
};

template <class S> struct b2dRot
{
	S c, s;
};

template <class S> struct b2dXf
{
	b2dVec2<S> p;
	b2dRot<S> q;
};
