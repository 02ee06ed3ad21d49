/*
 * CPU oracle for the BC7 block encoder -- the OPTION_PCA error bound (test
 * infrastructure only; see port_tables.h).
 *
 * Restates reference src/Bc7PcaEigen.cpp:26-146 (PrincipalComponentAnalysis<C>)
 * and :152-163 (InitPCA).  The reference computes the principal axis with
 * the third-party Eigen 3.3.7 (JacobiSVD with the Householder-QR
 * preconditioner, thin V; src/Bc7PcaEigen.cpp:72), which is not in the
 * reference tree, so this bound's parity with a PCA build of the reference
 * is unpinned: the SVD below restates Eigen's published algorithm (scale by
 * the largest magnitude; Householder QR of the tall matrix; two-sided
 * Jacobi sweeps over index pairs (p, q), q < p, with the 2x2 real SVD of
 * real_2x2_jacobi_svd and the symmetric Jacobi rotation of makeJacobi, until
 * every off-diagonal entry is within 2 eps of the largest diagonal one;
 * singular values made positive and sorted in descending order), with its
 * sums in the plain left-to-right order written here.  The CUDA encoder
 * runs the same float operations in the same order (nebc7_gb300/csrc/
 * bc7_pca.cuh) and is tested bit-exact against this.  The steps outside
 * the SVD keep the reference's operation order, with its fused multiply-
 * subtract (OPTION_FMA, on with AVX2, src/Bc7Mode.h:33-35).
 */
#include "port_core.h"

#include <math.h>

namespace nebc7_oracle {

namespace {

struct Rot
{
	float c, s;
};

/* Rows p and q of the C x C matrix m (row-major, stride 4) rotated:
   x' = c x + s y, y' = -s x + c y (Eigen's apply_rotation_in_the_plane). */
void RotateRows(float m[4][4], int C, int p, int q, Rot j)
{
	for (int i = 0; i < C; i++)
	{
		const float x = m[p][i], y = m[q][i];
		m[p][i] = j.c * x + j.s * y;
		m[q][i] = -j.s * x + j.c * y;
	}
}

/* Columns p and q rotated by the transpose of j (applyOnTheRight). */
void RotateCols(float m[4][4], int C, int p, int q, Rot j)
{
	const Rot t{ j.c, -j.s };
	for (int i = 0; i < C; i++)
	{
		const float x = m[i][p], y = m[i][q];
		m[i][p] = t.c * x + t.s * y;
		m[i][q] = -t.s * x + t.c * y;
	}
}

/* Eigen's JacobiRotation::makeJacobi for the symmetric [x y; y z]. */
Rot MakeJacobi(float x, float y, float z)
{
	const float deno = 2.0f * fabsf(y);
	if (deno < 1.17549435e-38f)
		return Rot{ 1.0f, 0.0f };
	const float tau = (x - z) / deno;
	const float w = sqrtf(tau * tau + 1.0f);
	const float t = tau > 0.0f ? 1.0f / (tau + w) : 1.0f / (tau - w);
	const float signT = t > 0.0f ? 1.0f : -1.0f;
	const float n = 1.0f / sqrtf(t * t + 1.0f);
	return Rot{ n, -signT * (y / fabsf(y)) * fabsf(t) * n };
}

/* Eigen's real_2x2_jacobi_svd: rotations with left * [pp pq; qp qq] * right diagonal. */
void Jacobi2x2(const float m[4][4], int p, int q, Rot* left, Rot* right)
{
	float a = m[p][p], b = m[p][q], c = m[q][p], d = m[q][q];
	Rot rot1;
	const float t = a + d;
	const float dd = c - b;
	if (fabsf(dd) < 1.17549435e-38f)
		rot1 = Rot{ 1.0f, 0.0f };
	else
	{
		const float u = t / dd;
		const float tmp = sqrtf(1.0f + u * u);
		rot1 = Rot{ u / tmp, 1.0f / tmp };
	}
	/* rot1 applied on the left of the 2x2 block */
	const float a1 = rot1.c * a + rot1.s * c, b1 = rot1.c * b + rot1.s * d;
	const float d1 = -rot1.s * b + rot1.c * d;
	*right = MakeJacobi(a1, b1, d1);
	/* left = rot1 * right^T */
	const Rot rt{ right->c, -right->s };
	*left = Rot{ rot1.c * rt.c - rot1.s * rt.s, rot1.c * rt.s + rot1.s * rt.c };
}

/* The first right singular vector (of the largest singular value) of the
   R x C matrix a (row-major, 4 floats per row), R >= C. */
void PrincipalAxis(float a[16][4], int R, int C, float v0[4])
{
	float scale = 0.0f;
	for (int j = 0; j < R; j++)
		for (int i = 0; i < C; i++)
			scale = fmaxf(scale, fabsf(a[j][i]));
	if (scale == 0.0f)
		scale = 1.0f;
	float w[4][4] = {};
	if (R != C)
	{
		/* Householder QR of a / scale (Eigen's householder_qr_inplace_unblocked) */
		float m[16][4];
		for (int j = 0; j < R; j++)
			for (int i = 0; i < C; i++)
				m[j][i] = a[j][i] / scale;
		for (int k = 0; k < C; k++)
		{
			/* makeHouseholder of column k, rows k..R-1 */
			float tailSq = 0.0f;
			for (int j = k + 1; j < R; j++)
				tailSq += m[j][k] * m[j][k];
			const float c0 = m[k][k];
			float tau, beta;
			float ess[16];
			if (tailSq <= 1.17549435e-38f)
			{
				tau = 0.0f;
				beta = c0;
				for (int j = k + 1; j < R; j++)
					ess[j] = 0.0f;
			}
			else
			{
				beta = sqrtf(c0 * c0 + tailSq);
				if (c0 >= 0.0f)
					beta = -beta;
				for (int j = k + 1; j < R; j++)
					ess[j] = m[j][k] / (c0 - beta);
				tau = (beta - c0) / beta;
			}
			m[k][k] = beta;
			for (int j = k + 1; j < R; j++)
				m[j][k] = ess[j];
			/* H applied on the left of the columns k+1.. (applyHouseholderOnTheLeft) */
			if (tau != 0.0f)
				for (int i = k + 1; i < C; i++)
				{
					float tmp = 0.0f;
					for (int j = k + 1; j < R; j++)
						tmp += ess[j] * m[j][i];
					tmp += m[k][i];
					m[k][i] -= tau * tmp;
					for (int j = k + 1; j < R; j++)
						m[j][i] -= tau * ess[j] * tmp;
				}
		}
		/* the work matrix: the upper triangle of R */
		for (int j = 0; j < C; j++)
			for (int i = 0; i < C; i++)
				w[j][i] = i >= j ? m[j][i] : 0.0f;
	}
	else
	{
		for (int j = 0; j < C; j++)
			for (int i = 0; i < C; i++)
				w[j][i] = a[j][i] / scale;
	}
	float V[4][4] = {};
	for (int i = 0; i < C; i++)
		V[i][i] = 1.0f;

	const float precision = 2.0f * 1.1920929e-7f;
	const float considerAsZero = 1.17549435e-38f;
	float maxDiag = 0.0f;
	for (int i = 0; i < C; i++)
		maxDiag = fmaxf(maxDiag, fabsf(w[i][i]));
	/* sweeps until no off-diagonal pair exceeds the threshold; a float matrix
	   of this size converges in a few sweeps (bounded here at 64) */
	for (int sweep = 0; sweep < 64; sweep++)
	{
		bool finished = true;
		for (int p = 1; p < C; p++)
			for (int q = 0; q < p; q++)
			{
				const float threshold = fmaxf(considerAsZero, precision * maxDiag);
				if (fabsf(w[p][q]) > threshold || fabsf(w[q][p]) > threshold)
				{
					finished = false;
					Rot jl, jr;
					Jacobi2x2(w, p, q, &jl, &jr);
					RotateRows(w, C, p, q, jl);
					RotateCols(w, C, p, q, jr);
					RotateCols(V, C, p, q, jr);
					maxDiag = fmaxf(maxDiag, fmaxf(fabsf(w[p][p]), fabsf(w[q][q])));
				}
			}
		if (finished)
			break;
	}
	/* singular values |w_ii|; the column of the largest (first on ties) */
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

} // namespace

/* src/Bc7PcaEigen.cpp:26-146 for C = 3 (G, R, B) or 4 (A, G, R, B). */
int PcaBound(const Config& cfg, const Area& area, int C)
{
	const int R = int(area.active);
	if (R < C)
		return 0;
	const int w[4] = { cfg.wA, cfg.wG, cfg.wR, cfg.wB };
	/* InitPCA (src/Bc7PcaEigen.cpp:152-163) */
	float K[4], invK[4];
	for (int c = 0; c < 4; c++)
	{
		K[c] = sqrtf(float(w[c]));
		invK[c] = 1.0f / K[c];
	}
	int sum[4] = { 0, 0, 0, 0 };
	for (int j = 0; j < R; j++)
		for (int c = 0; c < 4; c++)
			sum[c] = (sum[c] + area.px[j][c]) & 0xFFFF;
	float mean[4];
	for (int c = 0; c < 4; c++)
		mean[c] = (float(sum[c]) * K[c]) / float(R);
	/* the centred, scaled rows: G, R, B (C = 3) or A, G, R, B */
	float x[16][4];
	float m[16][4];
	for (int j = 0; j < R; j++)
	{
		for (int c = 0; c < 4; c++)
			x[j][c] = fmaf(float(area.px[j][c]), K[c], -mean[c]);
		for (int i = 0; i < C; i++)
			m[j][i] = x[j][i + 4 - C];
	}
	float v0[4];
	PrincipalAxis(m, R, C, v0);
	float mu[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
	for (int i = 0; i < C; i++)
		mu[i + 4 - C] = v0[i];
	unsigned total[4] = { 0, 0, 0, 0 };
	for (int j = 0; j < R; j++)
	{
		float mx[4];
		for (int c = 0; c < 4; c++)
			mx[c] = c < 4 - C ? 0.0f : m[j][c - (4 - C)];
		float l[4];
		for (int c = 0; c < 4; c++)
			l[c] = mu[c] * mx[c];
		const float lambda = (l[0] + l[1]) + (l[3] + l[2]);
		for (int c = 0; c < 4; c++)
		{
			float e = ((lambda * mu[c]) - mx[c]) * invK[c];
			e = fabsf(e);
			e = e - 1.1f;
			e = e > 0.0f ? e : 0.0f;
			const int md = int(e);   /* truncation (cvttps) */
			uint32_t v = uint32_t(md);
			if (!cfg.denoise)
			{
				/* saturating byte-wise doubling (adds_epu8) */
				uint32_t r = 0;
				for (int b = 0; b < 4; b++)
				{
					const uint32_t by = (v >> (8 * b)) & 0xFF;
					r |= (by * 2 > 255 ? 255 : by * 2) << (8 * b);
				}
				v = r;
			}
			const int shift = cfg.denoise ? cfg.denoise : 1;
			const uint32_t lo = ((v & 0xFFFF) >> shift), hi = ((v >> 16) >> shift);
			const uint32_t sq = ((lo * lo) & 0xFFFF) | (((hi * hi) & 0xFFFF) << 16);   /* mullo_epi16 */
			total[c] += sq;
		}
	}
	unsigned r = 0;
	for (int c = 0; c < 4; c++)
		r += total[c] * unsigned(c < 4 - C ? 0 : w[c]);
	return int(r);
}

} // namespace nebc7_oracle
