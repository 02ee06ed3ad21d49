/*
 * BC7 block encoder for sm_103a -- the OPTION_PCA error bound of the full
 * searches (opt-in: nebc7_set_pca; off by default, as in the reference's
 * src/Bc7Mode.h:5).
 *
 * PrincipalComponentAnalysis<C> (src/Bc7PcaEigen.cpp:26-146) bounds the
 * error of an area by the residual of its pixels around their principal
 * axis: the centred pixels, each channel scaled by the square root of its
 * weight (InitPCA, :152-163), are decomposed by a singular value
 * decomposition whose first right singular vector is the axis.  The
 * reference takes the SVD from the third-party Eigen 3.3.7 (JacobiSVD with
 * the Householder-QR preconditioner, :72), which is not in the reference
 * tree; this file restates Eigen's published algorithm -- scaling by the
 * largest magnitude, Householder QR of the tall matrix, two-sided Jacobi
 * sweeps over index pairs (p, q), q < p, with real_2x2_jacobi_svd and
 * makeJacobi until every off-diagonal entry is within 2 eps of the largest
 * diagonal one, singular values sorted in descending order -- with plain
 * left-to-right sums.  Every float operation is written as an IEEE
 * round-to-nearest intrinsic (no contraction into fused multiply-adds
 * except the reference's own fused multiply-subtract), in the order of the
 * CPU restatement the tests compare it with; parity with a PCA build of the
 * reference is unpinned.
 *
 * The bound is one lane's sequential work, once per area of a full search
 * of modes 1, 3, 6 and 7.
 */
#pragma once

#include "bc7_block.cuh"

namespace nebc7 {

namespace pca {

constexpr float kMinNormal = 1.17549435e-38f;
constexpr float kEps = 1.1920929e-7f;

struct Rot
{
	float c, s;
};

__device__ __forceinline__ float Mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float Add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float Sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float Div(float a, float b) { return __fdiv_rn(a, b); }

/* c x + s y and -s x + c y (Eigen's apply_rotation_in_the_plane). */
__device__ __forceinline__ void Rotate(float& x, float& y, Rot j)
{
	const float nx = Add(Mul(j.c, x), Mul(j.s, y));
	const float ny = Add(Mul(-j.s, x), Mul(j.c, y));
	x = nx;
	y = ny;
}

__device__ __forceinline__ Rot MakeJacobi(float x, float y, float z)
{
	const float deno = Mul(2.0f, fabsf(y));
	if (deno < kMinNormal)
		return Rot{ 1.0f, 0.0f };
	const float tau = Div(Sub(x, z), deno);
	const float w = __fsqrt_rn(Add(Mul(tau, tau), 1.0f));
	const float t = tau > 0.0f ? Div(1.0f, Add(tau, w)) : Div(1.0f, Sub(tau, w));
	const float signT = t > 0.0f ? 1.0f : -1.0f;
	const float n = Div(1.0f, __fsqrt_rn(Add(Mul(t, t), 1.0f)));
	return Rot{ n, Mul(Mul(Mul(-signT, Div(y, fabsf(y))), fabsf(t)), n) };
}

__device__ __forceinline__ void Jacobi2x2(const float m[4][4], int p, int q, Rot* left, Rot* right)
{
	const float a = m[p][p], b = m[p][q], c = m[q][p], d = m[q][q];
	Rot rot1;
	const float t = Add(a, d);
	const float dd = Sub(c, b);
	if (fabsf(dd) < kMinNormal)
		rot1 = Rot{ 1.0f, 0.0f };
	else
	{
		const float u = Div(t, dd);
		const float tmp = __fsqrt_rn(Add(1.0f, Mul(u, u)));
		rot1 = Rot{ Div(u, tmp), Div(1.0f, tmp) };
	}
	const float a1 = Add(Mul(rot1.c, a), Mul(rot1.s, c));
	const float b1 = Add(Mul(rot1.c, b), Mul(rot1.s, d));
	const float d1 = Add(Mul(-rot1.s, b), Mul(rot1.c, d));
	*right = MakeJacobi(a1, b1, d1);
	const Rot rt{ right->c, -right->s };
	*left = Rot{ Sub(Mul(rot1.c, rt.c), Mul(rot1.s, rt.s)), Add(Mul(rot1.c, rt.s), Mul(rot1.s, rt.c)) };
}

/* The first right singular vector of the R x C matrix a, R >= C. */
__device__ inline __noinline__ void PrincipalAxis(float a[16][4], int R, int C, float v0[4])
{
	float scale = 0.0f;
	for (int j = 0; j < R; j++)
		for (int i = 0; i < C; i++)
			scale = fmaxf(scale, fabsf(a[j][i]));
	if (scale == 0.0f)
		scale = 1.0f;
	float w[4][4];
	for (int j = 0; j < 4; j++)
		for (int i = 0; i < 4; i++)
			w[j][i] = 0.0f;
	if (R != C)
	{
		float m[16][4];
		for (int j = 0; j < R; j++)
			for (int i = 0; i < C; i++)
				m[j][i] = Div(a[j][i], scale);
		for (int k = 0; k < C; k++)
		{
			float tailSq = 0.0f;
			for (int j = k + 1; j < R; j++)
				tailSq = Add(tailSq, Mul(m[j][k], m[j][k]));
			const float c0 = m[k][k];
			float tau, beta;
			float ess[16];
			if (tailSq <= kMinNormal)
			{
				tau = 0.0f;
				beta = c0;
				for (int j = k + 1; j < R; j++)
					ess[j] = 0.0f;
			}
			else
			{
				beta = __fsqrt_rn(Add(Mul(c0, c0), tailSq));
				if (c0 >= 0.0f)
					beta = -beta;
				for (int j = k + 1; j < R; j++)
					ess[j] = Div(m[j][k], Sub(c0, beta));
				tau = Div(Sub(beta, c0), beta);
			}
			m[k][k] = beta;
			for (int j = k + 1; j < R; j++)
				m[j][k] = ess[j];
			if (tau != 0.0f)
				for (int i = k + 1; i < C; i++)
				{
					float tmp = 0.0f;
					for (int j = k + 1; j < R; j++)
						tmp = Add(tmp, Mul(ess[j], m[j][i]));
					tmp = Add(tmp, m[k][i]);
					m[k][i] = Sub(m[k][i], Mul(tau, tmp));
					for (int j = k + 1; j < R; j++)
						m[j][i] = Sub(m[j][i], Mul(Mul(tau, ess[j]), tmp));
				}
		}
		for (int j = 0; j < C; j++)
			for (int i = 0; i < C; i++)
				w[j][i] = i >= j ? m[j][i] : 0.0f;
	}
	else
	{
		for (int j = 0; j < C; j++)
			for (int i = 0; i < C; i++)
				w[j][i] = Div(a[j][i], scale);
	}
	float V[4][4];
	for (int j = 0; j < 4; j++)
		for (int i = 0; i < 4; i++)
			V[j][i] = i == j ? 1.0f : 0.0f;
	const float precision = Mul(2.0f, kEps);
	float maxDiag = 0.0f;
	for (int i = 0; i < C; i++)
		maxDiag = fmaxf(maxDiag, fabsf(w[i][i]));
	for (int sweep = 0; sweep < 64; sweep++)
	{
		bool finished = true;
		for (int p = 1; p < C; p++)
			for (int q = 0; q < p; q++)
			{
				const float threshold = fmaxf(kMinNormal, Mul(precision, maxDiag));
				if (fabsf(w[p][q]) > threshold || fabsf(w[q][p]) > threshold)
				{
					finished = false;
					Rot jl, jr;
					Jacobi2x2(w, p, q, &jl, &jr);
					for (int i = 0; i < C; i++)
						Rotate(w[p][i], w[q][i], jl);
					const Rot t{ jr.c, -jr.s };
					for (int i = 0; i < C; i++)
						Rotate(w[i][p], w[i][q], t);
					for (int i = 0; i < C; i++)
						Rotate(V[i][p], V[i][q], t);
					maxDiag = fmaxf(maxDiag, fmaxf(fabsf(w[p][p]), fabsf(w[q][q])));
				}
			}
		if (finished)
			break;
	}
	int best = 0;
	float bestV = fabsf(w[0][0]);
	for (int i = 1; i < C; i++)
		if (fabsf(w[i][i]) > bestV)
		{
			bestV = fabsf(w[i][i]);
			best = i;
		}
	for (int i = 0; i < C; i++)
		v0[i] = V[i][best];
}

} // namespace pca

/* PrincipalComponentAnalysis<C> (src/Bc7PcaEigen.cpp:26-146) of the first
   ai.active pixels of ar: C = 3 over G, R, B, C = 4 over A, G, R, B.  Lane
   0 computes it; every lane returns it. */
template<int kD>
__device__ __noinline__ int PcaBound(const Area& ar, const AreaInfo& ai, const Params& P, int C, int lane)
{
	using namespace pca;
	int result = 0;
	const int R = ai.active;
	if (lane == 0 && R >= C)
	{
		const int w[4] = { P.wA, P.wG, P.wR, P.wB };
		float K[4], invK[4];
		for (int c = 0; c < 4; c++)
		{
			K[c] = __fsqrt_rn(__int2float_rn(w[c]));
			invK[c] = Div(1.0f, K[c]);
		}
		int sum[4] = { 0, 0, 0, 0 };
		for (int j = 0; j < R; j++)
			for (int c = 0; c < 4; c++)
				sum[c] = (sum[c] + ar.px[j][c]) & 0xFFFF;
		float mean[4];
		for (int c = 0; c < 4; c++)
			mean[c] = Div(Mul(__int2float_rn(sum[c]), K[c]), __int2float_rn(R));
		float m[16][4];
		for (int j = 0; j < R; j++)
			for (int i = 0; i < C; i++)
			{
				const int c = i + 4 - C;
				/* the reference's fused multiply-subtract (OPTION_FMA) */
				m[j][i] = __fmaf_rn(__int2float_rn(ar.px[j][c]), K[c], -mean[c]);
			}
		float v0[4];
		PrincipalAxis(m, R, C, v0);
		float mu[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
		for (int i = 0; i < C; i++)
			mu[i + 4 - C] = v0[i];
		unsigned total[4] = { 0, 0, 0, 0 };
		for (int j = 0; j < R; j++)
		{
			float mx[4], l[4];
			for (int c = 0; c < 4; c++)
			{
				mx[c] = c < 4 - C ? 0.0f : m[j][c - (4 - C)];
				l[c] = Mul(mu[c], mx[c]);
			}
			const float lambda = Add(Add(l[0], l[1]), Add(l[3], l[2]));
			for (int c = 0; c < 4; c++)
			{
				float e = Mul(Sub(Mul(lambda, mu[c]), mx[c]), invK[c]);
				e = fabsf(e);
				e = Sub(e, 1.1f);
				e = e > 0.0f ? e : 0.0f;
				unsigned v = unsigned(__float2int_rz(e));
				if (!kD)
				{
					unsigned r = 0;
					for (int b = 0; b < 4; b++)
					{
						const unsigned by = (v >> (8 * b)) & 0xFF;
						r |= (by * 2 > 255 ? 255u : by * 2) << (8 * b);
					}
					v = r;
				}
				const int shift = kD ? kD : 1;
				const unsigned lo = (v & 0xFFFF) >> shift, hi = (v >> 16) >> shift;
				total[c] += ((lo * lo) & 0xFFFF) | (((hi * hi) & 0xFFFF) << 16);
			}
		}
		unsigned r = 0;
		for (int c = 0; c < 4; c++)
			r += total[c] * unsigned(c < 4 - C ? 0 : w[c]);
		result = int(r);
	}
	return __shfl_sync(kFull, result, 0);
}

} // namespace nebc7
