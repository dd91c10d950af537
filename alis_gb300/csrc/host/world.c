/*
 * world.c -- grid geometry, coefficient tables and world lifecycle.
 *
 * Host half of the reference src/world.c.  The geometry (index ranges,
 * coordinates, Bloch phases) and the 1-D CPML / dt/ds tables must be
 * bit-identical to the reference, because every kernel consumes them;
 * each function names the reference lines whose arithmetic it keeps
 * (operation order and float/double promotions included).  Fields live in
 * HBM; the float*** arrays allocated here are the host mirrors
 * (calloc-backed, so untouched pages cost no memory).
 */
#include <string.h>
#include "engine.h"

/* --- coordinate <-> index maps (reference src/world.c:12-54) --- */

/* Nearest index of coordinate x for a monotone map index->coordinate:
 * a 16-step bisection from 0 followed by a +-1 nearest-neighbour fix-up
 * (reference src/world.c:12-25). */
static int nearestIndex(world W, float (*map)(world, float), float x)
{
	int i = 0;
	for (int b = 15; b >= 0; b--) {
		float y = map(W, i);
		if (x > y) i += 1u << b;
		if (x < y) i -= 1u << b;
	}
	float d = fabsf(x - map(W, i));
	if (fabsf(x - map(W, i + 1)) < d) i++;
	if (fabsf(x - map(W, i - 1)) < d) i--;
	return i;
}

/* Graded grid: uniform spacing ds inside [min, max], geometric growth with
 * ratio r outside for n cells, then uniform spacing m*ds
 * (reference src/world.c:27-42). */
static float gradedCoordinate(int m, float min, float max, float ds, float i)
{
	float d = 10;
	float iLo = min/ds-0.5, iHi = max/ds+0.5;
	float r = d/(d-1), rr;
	int n = floor((d*m-0.5*m-0.5)*logf(m)/(m-1)+0.5);
	do {
		rr = r;
		r = rr - (powf(rr,n)-(d*m-0.5*m-0.5)*logf(rr)-1)/(n*powf(rr,n-1)-(d*m-0.5*m-0.5)/rr);
	} while (fabsf(r-rr) > 1E-6);
	if (i>=iHi+n) return ds * (iHi + (d*m-0.5*m-0.5) + (i-iHi-n) * m);
	if (i<=iLo-n) return ds * (iLo - (d*m-0.5*m-0.5) + (i-iLo+n) * m);
	if (i>iHi) return ds * (iHi + (powf(r,i-iHi)-1) / logf(r));
	if (i<iLo) return ds * (iLo - (powf(r,iLo-i)-1) / logf(r));
	return ds * i;
}

static int xtoi(world W, float x) { return nearestIndex(W, W->itox, x); }
static int ytoj(world W, float y) { return nearestIndex(W, W->jtoy, y); }
static int ztok(world W, float z) { return nearestIndex(W, W->ktoz, z); }
static float itoxUniform(world W, float i) { return W->dx*i; }
static float jtoyUniform(world W, float j) { return W->dy*j; }
static float ktozUniform(world W, float k) { return W->dz*k; }
static float itoxGraded(world W, float i) { return gradedCoordinate(W->Res.nug.x.m, W->Res.nug.x.Min, W->Res.nug.x.Max, W->dx, i); }
static float jtoyGraded(world W, float j) { return gradedCoordinate(W->Res.nug.y.m, W->Res.nug.y.Min, W->Res.nug.y.Max, W->dy, j); }
static float ktozGraded(world W, float k) { return gradedCoordinate(W->Res.nug.z.m, W->Res.nug.z.Min, W->Res.nug.z.Max, W->dz, k); }


/* --- 3-D arrays with arbitrary index bases (reference src/world.c:58-85) --- */

/* One zeroed data block plus two row-pointer tables, so that
 * f[i][j][k] is valid for i in [i0,i1], j in [j0,j1], k in [k0,k1]. */
#define MAKE3D(T, f, i0, i1, j0, j1, k0, k1) do { \
	long ni_ = 1L-(i0)+(i1), nj_ = 1L-(j0)+(j1), nk_ = 1L-(k0)+(k1); \
	MALLOC(f, i0, ni_); \
	MALLOC(f[i0], j0, ni_*nj_); \
	MALLOC(f[i0][j0], k0, ni_*nj_*nk_); \
	for (long a_ = 0; a_ < ni_; a_++) { \
		f[(i0)+a_] = f[i0] + nj_*a_; \
		for (long b_ = 0; b_ < nj_; b_++) f[(i0)+a_][(j0)+b_] = f[i0][j0] + nk_*(nj_*a_+b_); \
	} \
} while (0)

float ***makeField(int iMin, int iMax, int jMin, int jMax, int kMin, int kMax)
{
	float ***f;
	MAKE3D(float, f, iMin, iMax, jMin, jMax, kMin, kMax);
	return f;
}

float complex ***makeComplexField(int iMin, int iMax, int jMin, int jMax, int kMin, int kMax)
{
	float complex ***f;
	MAKE3D(float complex, f, iMin, iMax, jMin, jMax, kMin, kMax);
	return f;
}

static void zeroField(float ***f, int iMin, int iMax, int jMin, int jMax, int kMin, int kMax)
{
	if (!f) return;
	size_t n = (size_t)(1-iMin+iMax)*(1-jMin+jMax)*(1-kMin+kMax);
	memset(&f[iMin][jMin][kMin], 0, n*sizeof(float));
}


/* --- CPML and spacing tables (reference src/world.c:98-161) --- */

/* Grading of sigma, kappa, alpha over the Num cells of a PML face, the
 * kappa-stretched dt/ds, and the psi recursion coefficients
 * C0 = (1-x)/(1+x), C1,C2 = -/+ dt/ds * sigma dt/ds / (1+x)
 * with x = (sigma dt/ds + alpha dt)/2 (reference src/world.c:98-132). */
static void cpmlTables(sur S, int Offset, float **C0, float **C1, float **C2, float *dtds, float dt,
                       int MinSur, int MaxSur, int Min, int Max, int MIN, int NUM)
{
	if (!S.pml.SigmaMax) S.pml.SigmaMax = 1;
	if (!S.pml.KappaMax) S.pml.KappaMax = S.pml.Num < 24 ? 1 : 10;
	if (!S.pml.AlphaMax) S.pml.AlphaMax = S.pml.Num < 24 ? 0 : 0.01;
	if (!S.pml.SigmaPower) S.pml.SigmaPower = 3.5;
	if (!S.pml.AlphaPower) S.pml.AlphaPower = 1;
	if (MinSur != PML && MaxSur != PML) return;
	MALLOC(*C0, MIN, NUM);
	MALLOC(*C1, MIN, NUM);
	MALLOC(*C2, MIN, NUM);
	for (int n = 1; n <= S.pml.Num; n++) {
		float Sigma = 0.8*S.pml.SigmaMax*(S.pml.SigmaPower+1)*powf((n-0.5*Offset)/S.pml.Num, S.pml.SigmaPower);
		float Kappa = 1+(S.pml.KappaMax-1)*powf((n-0.5*Offset)/S.pml.Num, S.pml.SigmaPower);
		float Alpha = S.pml.AlphaMax*powf((S.pml.Num-(n-0.5*Offset))/S.pml.Num, S.pml.AlphaPower);
		int side[2] = { Min-n-1+Offset, Max+n+1 };
		int use[2] = { MinSur==PML, MaxSur==PML };
		for (int s = 0; s < 2; s++) {
			if (!use[s]) continue;
			int q = side[s];
			dtds[q] /= Kappa;
			float Ca = (1-0.5*(Sigma*dtds[q]+Alpha*dt))/(1+0.5*(Sigma*dtds[q]+Alpha*dt));
			float Cb = Sigma*dtds[q]/(1+0.5*(Sigma*dtds[q]+Alpha*dt));
			(*C0)[q] = Ca;
			(*C1)[q] = -dtds[q]*Cb;
			(*C2)[q] = +dtds[q]*Cb;
		}
	}
}

/* Spacing and dt/ds tables of the E grid (Offset 0, cells centred on i)
 * or the H grid (Offset 1, cells between i-1 and i) (reference
 * src/world.c:135-161). */
static coeffs *spacingTables(world W, sur S, int Offset)
{
	coeffs *C;
	MALLOC(C, 0, 1);
	S.pml.Num = S.pml.Num ? S.pml.Num : 12;
	int symx = W->xMinSur==SYM, symy = W->yMinSur==SYM, symz = W->zMinSur==SYM;
	MALLOC(C->dx, symx ? -W->iMAX : W->iMIN, symx ? 2*W->iNUM-1 : W->iNUM);
	MALLOC(C->dy, symy ? -W->jMAX : W->jMIN, symy ? 2*W->jNUM-1 : W->jNUM);
	MALLOC(C->dz, symz ? -W->kMAX : W->kMIN, symz ? 2*W->kNUM-1 : W->kNUM);
	MALLOC(C->dtdx, W->iMIN, W->iNUM);
	MALLOC(C->dtdy, W->jMIN, W->jNUM);
	MALLOC(C->dtdz, W->kMIN, W->kNUM);
	for (int i = W->iMIN; i <= W->iMAX; i++)
		C->dtdx[i] = W->dt/(C->dx[i]=(W->itox(W, i-0.5*(Offset-1))-W->itox(W, i-0.5*(Offset+1))));
	for (int j = W->jMIN; j <= W->jMAX; j++)
		C->dtdy[j] = W->dt/(C->dy[j]=(W->jtoy(W, j-0.5*(Offset-1))-W->jtoy(W, j-0.5*(Offset+1))));
	for (int k = W->kMIN; k <= W->kMAX; k++)
		C->dtdz[k] = W->dt/(C->dz[k]=(W->ktoz(W, k-0.5*(Offset-1))-W->ktoz(W, k-0.5*(Offset+1))));
	if (symx) for (int i = 1; i <= W->iMAX; i++) C->dx[-i] = C->dx[i];
	if (symy) for (int j = 1; j <= W->jMAX; j++) C->dy[-j] = C->dy[j];
	if (symz) for (int k = 1; k <= W->kMAX; k++) C->dz[-k] = C->dz[k];
	cpmlTables(S, Offset, &C->xP, &C->xPy, &C->xPz, C->dtdx, W->dt, W->xMinSur, W->xMaxSur, W->iMin, W->iMax, W->iMIN, W->iNUM);
	cpmlTables(S, Offset, &C->yP, &C->yPz, &C->yPx, C->dtdy, W->dt, W->yMinSur, W->yMaxSur, W->jMin, W->jMax, W->jMIN, W->jNUM);
	cpmlTables(S, Offset, &C->zP, &C->zPx, &C->zPy, C->dtdz, W->dt, W->zMinSur, W->zMaxSur, W->kMin, W->kMax, W->kMIN, W->kNUM);
	C->N = 0;
	return C;
}


/* --- field containers (reference src/world.c:164-189) --- */

/* psi slab of face `face` (0..5 = xMin,yMin,zMin,xMax,yMax,zMax) for the
 * E (Offset 0) or H (Offset 1) grid; ranges follow reference
 * src/world.c:174-186. */
void alis_psi_range(world W, int face, int Offset, int r[6])
{
	int a[6] = { W->iMIN, W->iMAX, W->jMIN, W->jMAX, W->kMIN, W->kMAX };
	int mins[3] = { W->iMin, W->jMin, W->kMin }, maxs[3] = { W->iMax, W->jMax, W->kMax };
	int MINs[3] = { W->iMIN, W->jMIN, W->kMIN }, MAXs[3] = { W->iMAX, W->jMAX, W->kMAX };
	int d = face % 3;
	for (int q = 0; q < 6; q++) r[q] = a[q];
	if (face < 3) r[2*d] = MINs[d]+Offset, r[2*d+1] = mins[d]+Offset-2;
	else r[2*d] = maxs[d]+2, r[2*d+1] = MAXs[d];
}

static int facePML(world W, int face)
{
	int s[6] = { W->xMinSur, W->yMinSur, W->zMinSur, W->xMaxSur, W->yMaxSur, W->zMaxSur };
	return s[face] == PML;
}

/* pointer slots of the two psi arrays of each face: xMin -> (Py, Pz),
 * yMin -> (Pz, Px), zMin -> (Px, Py), same for the max faces. */
float ****alis_psi_slot(vfield *F, int face, int which)
{
	float ****t[6][2] = {
		{ &F->xMinPy, &F->xMinPz }, { &F->yMinPz, &F->yMinPx }, { &F->zMinPx, &F->zMinPy },
		{ &F->xMaxPy, &F->xMaxPz }, { &F->yMaxPz, &F->yMaxPx }, { &F->zMaxPx, &F->zMaxPy } };
	return t[face][which];
}

static vfield *makeFields(world W, int Offset)
{
	vfield *F;
	MALLOC(F, 0, 1+W->complexField);
	for (int m = 0; m <= W->complexField; m++) {
		F[m].x = makeField(W->iMIN-1, W->iMAX+1, W->jMIN-1, W->jMAX+1, W->kMIN-1, W->kMAX+1);
		F[m].y = makeField(W->iMIN-1, W->iMAX+1, W->jMIN-1, W->jMAX+1, W->kMIN-1, W->kMAX+1);
		F[m].z = makeField(W->iMIN-1, W->iMAX+1, W->jMIN-1, W->jMAX+1, W->kMIN-1, W->kMAX+1);
		for (int face = 0; face < 6; face++) {
			if (!facePML(W, face)) continue;
			int r[6];
			alis_psi_range(W, face, Offset, r);
			for (int w = 0; w < 2; w++) *alis_psi_slot(&F[m], face, w) = makeField(r[0], r[1], r[2], r[3], r[4], r[5]);
		}
	}
	return F;
}


/* --- world lifecycle (reference src/world.c:192-280, 318-466) --- */

static world newWorldGeometry(res R, dom D, sur S)
{
	world W;
	MALLOC(W, 0, 1);

	/* symmetric graded-grid core, Bloch from PBC with a period, PML default */
	if (R.nug.x.Min>0) R.nug.x.Max = R.nug.x.Min, R.nug.x.Min = -R.nug.x.Max;
	if (R.nug.y.Min>0) R.nug.y.Max = R.nug.y.Min, R.nug.y.Min = -R.nug.y.Max;
	if (R.nug.z.Min>0) R.nug.z.Max = R.nug.z.Min, R.nug.z.Min = -R.nug.z.Max;
	if (S.x.MinSur==PBC && S.x.MaxSur) S.x.MinSur=BBC;
	if (S.y.MinSur==PBC && S.y.MaxSur) S.y.MinSur=BBC;
	if (S.z.MinSur==PBC && S.z.MaxSur) S.z.MinSur=BBC;
	if (!S.pml.Num) S.pml.Num = 12;

	*W = (struct world) { D, R, S, 0, R.dt, R.d.x, R.d.y?R.d.y:R.d.x, R.d.z?R.d.z:R.d.x, R.spec.eV?R.spec.eV:1, INF };
	/* {a} means [-a, a]; a symmetry plane mirrors the domain */
	if ((!D.x.Max && D.x.Min>0) || S.x.MinSur==SYM) D.x.Min = -(D.x.Max = D.x.Max ? D.x.Max : D.x.Min);
	if ((!D.y.Max && D.y.Min>0) || S.y.MinSur==SYM) D.y.Min = -(D.y.Max = D.y.Max ? D.y.Max : D.y.Min);
	if ((!D.z.Max && D.z.Min>0) || S.z.MinSur==SYM) D.z.Min = -(D.z.Max = D.z.Max ? D.z.Max : D.z.Min);

	W->itox = R.gridFunction.itox ? R.gridFunction.itox : R.nug.x.m > 1 ? itoxGraded : itoxUniform;
	W->jtoy = R.gridFunction.jtoy ? R.gridFunction.jtoy : R.nug.y.m > 1 ? jtoyGraded : jtoyUniform;
	W->ktoz = R.gridFunction.ktoz ? R.gridFunction.ktoz : R.nug.z.m > 1 ? ktozGraded : ktozUniform;
	W->xtoi = xtoi, W->ytoj = ytoj, W->ztok = ztok;

	/* y and z inherit x's boundary when left unset; a Bloch min side
	 * carries the period in MaxSur, so the max side copies the min side */
	W->xMinSur = S.x.MinSur;
	W->yMinSur = S.y.MinSur ? S.y.MinSur : S.x.MinSur;
	W->zMinSur = S.z.MinSur ? S.z.MinSur : S.x.MinSur;
	W->xMaxSur = S.x.MinSur!=BBC && S.x.MaxSur ? S.x.MaxSur : S.x.MinSur;
	W->yMaxSur = S.y.MinSur!=BBC && S.y.MaxSur ? S.y.MaxSur : S.y.MinSur ? S.y.MinSur : S.x.MinSur;
	W->zMaxSur = S.z.MinSur!=BBC && S.z.MaxSur ? S.z.MaxSur : S.z.MinSur ? S.z.MinSur : S.x.MinSur;

	W->iMin = W->xMinSur==SYM ? 0 : D.x.Min || D.x.Max ? W->xtoi(W, D.x.Min) : -1;
	W->jMin = W->yMinSur==SYM ? 0 : D.y.Min || D.y.Max ? W->ytoj(W, D.y.Min) : -1;
	W->kMin = W->zMinSur==SYM ? 0 : D.z.Min || D.z.Max ? W->ztok(W, D.z.Min) : -1;
	W->iMax = D.x.Min || D.x.Max ? W->xtoi(W, D.x.Max) : 1, W->iNum = 1-W->iMin+W->iMax;
	W->jMax = D.y.Min || D.y.Max ? W->ytoj(W, D.y.Max) : 1, W->jNum = 1-W->jMin+W->jMax;
	W->kMax = D.z.Min || D.z.Max ? W->ztok(W, D.z.Max) : 1, W->kNum = 1-W->kMin+W->kMax;

	/* PML cells are added outside the domain: Num+1 per PML face */
	W->iMIN = W->iMin-(W->xMinSur==PML ? S.pml.Num+1 : 0);
	W->jMIN = W->jMin-(W->yMinSur==PML ? S.pml.Num+1 : 0);
	W->kMIN = W->kMin-(W->zMinSur==PML ? S.pml.Num+1 : 0);
	W->iMAX = W->iMax+(W->xMaxSur==PML ? S.pml.Num+1 : 0), W->iNUM = 1-W->iMIN+W->iMAX;
	W->jMAX = W->jMax+(W->yMaxSur==PML ? S.pml.Num+1 : 0), W->jNUM = 1-W->jMIN+W->jMAX;
	W->kMAX = W->kMax+(W->zMaxSur==PML ? S.pml.Num+1 : 0), W->kNUM = 1-W->kMIN+W->kMAX;

	W->xMax = W->itox(W, W->iMax), W->xMin = W->xMinSur==SYM ? -W->xMax : W->itox(W, W->iMin), W->xSize = W->xMax - W->xMin;
	W->yMax = W->jtoy(W, W->jMax), W->yMin = W->yMinSur==SYM ? -W->yMax : W->jtoy(W, W->jMin), W->ySize = W->yMax - W->yMin;
	W->zMax = W->ktoz(W, W->kMax), W->zMin = W->zMinSur==SYM ? -W->zMax : W->ktoz(W, W->kMin), W->zSize = W->zMax - W->zMin;
	W->xMAX = W->itox(W, W->iMAX), W->xMIN = W->xMinSur==SYM ? -W->xMAX : W->itox(W, W->iMIN);
	W->yMAX = W->jtoy(W, W->jMAX), W->yMIN = W->yMinSur==SYM ? -W->yMAX : W->jtoy(W, W->jMIN);
	W->zMAX = W->ktoz(W, W->kMAX), W->zMIN = W->zMinSur==SYM ? -W->zMAX : W->ktoz(W, W->kMIN);

	/* Bloch phase across one period; a symmetry plane starts at cos = 0
	 * until a source fixes its parity (reference src/world.c:243-253) */
	int bx = S.x.MinSur==BBC && S.x.MaxSur, by = S.y.MinSur==BBC && S.y.MaxSur, bz = S.z.MinSur==BBC && S.z.MaxSur;
	W->coskx = bx ? cosf(2*PI*(W->xMax-W->xMin)/S.x.MaxSur) : S.x.MinSur==SYM ? 0 : 1;
	W->cosky = by ? cosf(2*PI*(W->yMax-W->yMin)/S.y.MaxSur) : S.y.MinSur==SYM ? 0 : 1;
	W->coskz = bz ? cosf(2*PI*(W->zMax-W->zMin)/S.z.MaxSur) : S.z.MinSur==SYM ? 0 : 1;
	W->sinkx = bx ? sinf(2*PI*(W->xMax-W->xMin)/S.x.MaxSur) : 0;
	W->sinky = by ? sinf(2*PI*(W->yMax-W->yMin)/S.y.MaxSur) : 0;
	W->sinkz = bz ? sinf(2*PI*(W->zMax-W->zMin)/S.z.MaxSur) : 0;
	int hb = S.y.MinSur==HBC && S.y.MaxSur;
	W->coskyp = hb ? cosf(PI*(2*(W->yMax-W->yMin)/S.y.MaxSur+(W->xMax-W->xMin)/S.x.MaxSur)) : 1;
	W->coskym = hb ? cosf(PI*(2*(W->yMax-W->yMin)/S.y.MaxSur-(W->xMax-W->xMin)/S.x.MaxSur)) : 1;
	W->sinkyp = hb ? sinf(PI*(2*(W->yMax-W->yMin)/S.y.MaxSur+(W->xMax-W->xMin)/S.x.MaxSur)) : 0;
	W->sinkym = hb ? sinf(PI*(2*(W->yMax-W->yMin)/S.y.MaxSur-(W->xMax-W->xMin)/S.x.MaxSur)) : 0;

	W->xyArea = W->xSize * W->ySize, W->xzArea = W->xSize * W->zSize, W->yzArea = W->ySize * W->zSize;
	if (S.x.MinSur==BBC || S.y.MinSur==BBC || S.z.MinSur==BBC) W->complexField = 1;
	return W;
}

world createWorld(dom D, res R, sur S, char *format, ...)
{
	va_list ap;
	world W = newWorldGeometry(R, D, S);
	W->E = makeFields(W, 0);
	W->H = makeFields(W, 1);
	W->CE = spacingTables(W, S, 0);
	W->CH = spacingTables(W, S, 1);
	va_start(ap, format);
	vsnprintf(W->ID, sizeof W->ID, format, ap);
	va_end(ap);
	if (W->ID[0]) {
		/* start from a clean output set, as the reference does */
		printf("Deleting previous files.");
		exec("rm -fr %s %s.c?* %s[#--0-~]* %s.[#-bd-~]* 2> /dev/null", W->ID, W->ID, W->ID, W->ID);
	}
	alis_be_world_created(W);
	return W;
}

/* the per-object J/K containers of an E field set (reference
 * src/world.c:283-315 and src/object.c:207-225) */
void alis_make_currents(world W, vfield *F, coeffs *C, int n)
{
	for (int m = 0; m <= W->complexField; m++) {
		MALLOC(F[m].Jx[n], 0, C->NK[n]);
		MALLOC(F[m].Jy[n], 0, C->NK[n]);
		MALLOC(F[m].Jz[n], 0, C->NK[n]);
		MALLOC(F[m].Kx[n], C->NJ[n], C->NK[n] - C->NJ[n]);
		MALLOC(F[m].Ky[n], C->NJ[n], C->NK[n] - C->NJ[n]);
		MALLOC(F[m].Kz[n], C->NJ[n], C->NK[n] - C->NJ[n]);
		for (int p = 0; p < C->NK[n]; p++) {
			F[m].Jx[n][p] = makeField(C->iMin[n], C->iMax[n], C->jMin[n], C->jMax[n], C->kMin[n], C->kMax[n]);
			F[m].Jy[n][p] = makeField(C->iMin[n], C->iMax[n], C->jMin[n], C->jMax[n], C->kMin[n], C->kMax[n]);
			F[m].Jz[n][p] = makeField(C->iMin[n], C->iMax[n], C->jMin[n], C->jMax[n], C->kMin[n], C->kMax[n]);
		}
		for (int p = C->NJ[n]; p < C->NK[n]; p++) {
			F[m].Kx[n][p] = makeField(C->iMin[n], C->iMax[n], C->jMin[n], C->jMax[n], C->kMin[n], C->kMax[n]);
			F[m].Ky[n][p] = makeField(C->iMin[n], C->iMax[n], C->jMin[n], C->jMax[n], C->kMin[n], C->kMax[n]);
			F[m].Kz[n][p] = makeField(C->iMin[n], C->iMax[n], C->jMin[n], C->jMax[n], C->kMin[n], C->kMax[n]);
		}
	}
}

void alis_alloc_current_tables(world W, vfield *F, int N)
{
	for (int m = 0; m <= W->complexField; m++) {
		MALLOC(F[m].Jx, 0, N); MALLOC(F[m].Jy, 0, N); MALLOC(F[m].Jz, 0, N);
		MALLOC(F[m].Kx, 0, N); MALLOC(F[m].Ky, 0, N); MALLOC(F[m].Kz, 0, N);
	}
}

world cloneWorld(world SW)
{
	world W;
	MALLOC(W, 0, 1);
	*W = *SW;
	W->E = makeFields(W, 0);
	W->H = makeFields(W, 1);
	coeffs *C = W->CE;
	alis_alloc_current_tables(W, W->E, C->N);
	alis_alloc_current_tables(W, W->H, W->CH->N);
	for (int n = 0; n < C->N; n++) alis_make_currents(W, W->E, C, n);
	alis_be_world_created(W);
	alis_be_objects_changed(W);
	alis_be_sources_changed(W);
	return W;
}

static void zeroVectorField(world W, vfield *F, coeffs *C, int Offset)
{
	for (int m = 0; m <= W->complexField; m++) {
		zeroField(F[m].x, W->iMIN-1, W->iMAX+1, W->jMIN-1, W->jMAX+1, W->kMIN-1, W->kMAX+1);
		zeroField(F[m].y, W->iMIN-1, W->iMAX+1, W->jMIN-1, W->jMAX+1, W->kMIN-1, W->kMAX+1);
		zeroField(F[m].z, W->iMIN-1, W->iMAX+1, W->jMIN-1, W->jMAX+1, W->kMIN-1, W->kMAX+1);
		for (int face = 0; face < 6; face++) {
			int r[6];
			alis_psi_range(W, face, Offset, r);
			for (int w = 0; w < 2; w++) zeroField(*alis_psi_slot(&F[m], face, w), r[0], r[1], r[2], r[3], r[4], r[5]);
		}
		for (int n = 0; n < C->N; n++) {
			for (int p = 0; p < C->NK[n]; p++) {
				zeroField(F[m].Jx[n][p], C->iMin[n], C->iMax[n], C->jMin[n], C->jMax[n], C->kMin[n], C->kMax[n]);
				zeroField(F[m].Jy[n][p], C->iMin[n], C->iMax[n], C->jMin[n], C->jMax[n], C->kMin[n], C->kMax[n]);
				zeroField(F[m].Jz[n][p], C->iMin[n], C->iMax[n], C->jMin[n], C->jMax[n], C->kMin[n], C->kMax[n]);
			}
			for (int p = C->NJ[n]; p < C->NK[n]; p++) {
				zeroField(F[m].Kx[n][p], C->iMin[n], C->iMax[n], C->jMin[n], C->jMax[n], C->kMin[n], C->kMax[n]);
				zeroField(F[m].Ky[n][p], C->iMin[n], C->iMax[n], C->jMin[n], C->jMax[n], C->kMin[n], C->kMax[n]);
				zeroField(F[m].Kz[n][p], C->iMin[n], C->iMax[n], C->jMin[n], C->jMax[n], C->kMin[n], C->kMax[n]);
			}
		}
	}
}

void rebootWorld(world W)
{
	removeSources(W);
	zeroVectorField(W, W->E, W->CE, 0);
	zeroVectorField(W, W->H, W->CH, 1);
	W->t = W->E->t = 0;
	W->H->t = 0.5;
	W->n = 0;
	printf("\n");
	alis_be_world_reset(W);
}

void alis_free_currents(world W, vfield *F, coeffs *C)
{
	for (int m = 0; m <= W->complexField; m++) {
		for (int n = 0; n < C->N; n++) {
			for (int p = 0; p < C->NK[n]; p++) {
				removeField(F[m].Jx[n][p], C->iMin[n], C->jMin[n], C->kMin[n]);
				removeField(F[m].Jy[n][p], C->iMin[n], C->jMin[n], C->kMin[n]);
				removeField(F[m].Jz[n][p], C->iMin[n], C->jMin[n], C->kMin[n]);
			}
			for (int p = C->NJ[n]; p < C->NK[n]; p++) {
				removeField(F[m].Kx[n][p], C->iMin[n], C->jMin[n], C->kMin[n]);
				removeField(F[m].Ky[n][p], C->iMin[n], C->jMin[n], C->kMin[n]);
				removeField(F[m].Kz[n][p], C->iMin[n], C->jMin[n], C->kMin[n]);
			}
			free(F[m].Jx[n]); free(F[m].Kx[n]+C->NJ[n]);
			free(F[m].Jy[n]); free(F[m].Ky[n]+C->NJ[n]);
			free(F[m].Jz[n]); free(F[m].Kz[n]+C->NJ[n]);
		}
		free(F[m].Jx); free(F[m].Kx);
		free(F[m].Jy); free(F[m].Ky);
		free(F[m].Jz); free(F[m].Kz);
		F[m].Jx = F[m].Jy = F[m].Jz = F[m].Kx = F[m].Ky = F[m].Kz = 0;
	}
}

static void freeFields(world W, vfield *F, int Offset)
{
	for (int m = 0; m <= W->complexField; m++) {
		removeField(F[m].x, W->iMIN-1, W->jMIN-1, W->kMIN-1);
		removeField(F[m].y, W->iMIN-1, W->jMIN-1, W->kMIN-1);
		removeField(F[m].z, W->iMIN-1, W->jMIN-1, W->kMIN-1);
		for (int face = 0; face < 6; face++) {
			float ****slot;
			int r[6];
			alis_psi_range(W, face, Offset, r);
			for (int w = 0; w < 2; w++) {
				slot = alis_psi_slot(&F[m], face, w);
				if (*slot) removeField((*slot), r[0], r[2], r[4]);
			}
		}
	}
	free(F);
}

static void freeSpacingTables(world W, coeffs *C)
{
	if (C->xP) free(&C->xP[W->iMIN]), free(&C->xPy[W->iMIN]), free(&C->xPz[W->iMIN]);
	if (C->yP) free(&C->yP[W->jMIN]), free(&C->yPz[W->jMIN]), free(&C->yPx[W->jMIN]);
	if (C->zP) free(&C->zP[W->kMIN]), free(&C->zPx[W->kMIN]), free(&C->zPy[W->kMIN]);
	free(&C->dtdx[W->iMIN]), free(&C->dx[W->xMinSur!=SYM ? W->iMIN : -W->iMAX]);
	free(&C->dtdy[W->jMIN]), free(&C->dy[W->yMinSur!=SYM ? W->jMIN : -W->jMAX]);
	free(&C->dtdz[W->kMIN]), free(&C->dz[W->zMinSur!=SYM ? W->kMIN : -W->kMAX]);
	free(C);
}

void deleteWorld(world W)
{
	alis_be_world_deleted(W);
	removeSources(W);
	removeObjects(W);
	freeSpacingTables(W, W->CE);
	freeSpacingTables(W, W->CH);
	freeFields(W, W->E, 0);
	freeFields(W, W->H, 1);
	free(W);
}

void deleteCloneWorld(world W)
{
	alis_be_world_deleted(W);
	removeSources(W);
	alis_free_currents(W, W->E, W->CE);
	alis_free_currents(W, W->H, W->CH);
	freeFields(W, W->E, 0);
	freeFields(W, W->H, 1);
	free(W);
}

void alisSyncHost(world W)
{
	alis_be_sync_world(W);
	alis_be_sync_phasers_of(W);
}

void alisWorldStreams(world W)
{
	alis_be_world_streams(W);
}

void alisBatchBegin(void)
{
	alis_be_batch(1);
}

void alisBatchEnd(void)
{
	alis_be_batch(0);
}


/* --- HDF5 I/O (reference src/world.c:469-537) ---
 * libhdf5 is not part of this build; the two entry points exist so that
 * programs link, and fail loudly when called. */
void *h5read(int *dim, char *format, ...)
{
	(void)dim; (void)format;
	fprintf(stderr, "alis: h5read is unavailable (built without HDF5)\n");
	exit(1);
}

void h5write(int *dim, float *p, char *format, ...)
{
	(void)dim; (void)p; (void)format;
	fprintf(stderr, "alis: h5write is unavailable (built without HDF5)\n");
	exit(1);
}
