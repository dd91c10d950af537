/*
 * shapes.c -- point-membership predicates int S(object, x, y, z).
 *
 * Same geometry and the same float arithmetic as the reference
 * src/shapes.c (cited per shape), since the voxelized material maps must
 * match bit for bit.  An object's f[3][3] holds either a bounding box
 * {{xMin,xMax},{yMin,yMax},{zMin,zMax}} or, when f[2][0] == f[2][1], a
 * centre/half-size pair {{x0,y0,z0},{a,b,c}} (b and c default to a).
 * The compound shapes reference a nested object list through O.p.
 */
#include "engine.h"

/* Bounding box of a basic shape.  The centre form reproduces the
 * reference expression (src/shapes.c:9-12) exactly, including its
 * operator precedence: for y and z the test "x0 - a" (resp. "x0 + a")
 * selects between the two half-sizes instead of forming an offset. */
typedef struct { float xMin, xMax, yMin, yMax, zMin, zMax; } box;

static box bounds(object O)
{
	box b;
	if (O.f[2][1]-O.f[2][0]) {
		b.xMin = O.f[0][0], b.xMax = O.f[0][1];
		b.yMin = O.f[1][0], b.yMax = O.f[1][1];
		b.zMin = O.f[2][0], b.zMax = O.f[2][1];
	} else {
		b.xMin = O.f[0][0]-O.f[1][0];
		b.yMin = (O.f[0][1]-O.f[1][1]) ? O.f[1][1] : O.f[1][0];
		b.zMin = (O.f[0][2]-O.f[1][2]) ? O.f[1][2] : O.f[1][0];
		b.xMax = O.f[0][0]+O.f[1][0];
		b.yMax = (O.f[0][1]+O.f[1][1]) ? O.f[1][1] : O.f[1][0];
		b.zMax = (O.f[0][2]+O.f[1][2]) ? O.f[1][2] : O.f[1][0];
	}
	return b;
}

/* normalised coordinate in [-1, 1] across [lo, hi] */
#define U(v, lo, hi) ((2*(v)-(lo)-(hi))/((hi)-(lo)))
#define IN(v, lo, hi) ((lo) <= (v) && (v) <= (hi))
#define INOPEN(v, lo, hi) ((lo) < (v) && (v) < (hi))

/* reference src/shapes.c:17-21 */
int Box(object O, float x, float y, float z)
{
	box b = bounds(O);
	return IN(x, b.xMin, b.xMax) && IN(y, b.yMin, b.yMax) && IN(z, b.zMin, b.zMax);
}

/* ellipsoid, reference src/shapes.c:23-27 */
int Ball(object O, float x, float y, float z)
{
	box b = bounds(O);
	return sq(U(x, b.xMin, b.xMax))+sq(U(y, b.yMin, b.yMax))+sq(U(z, b.zMin, b.zMax)) < 1;
}

/* octahedron, reference src/shapes.c:29-33 */
int Diamond(object O, float x, float y, float z)
{
	box b = bounds(O);
	return fabsf(U(x, b.xMin, b.xMax))+fabsf(U(y, b.yMin, b.yMax))+fabsf(U(z, b.zMin, b.zMax)) <= 1;
}

/* double cones; the radial term is a double-precision sqrt
 * (reference src/shapes.c:35-51) */
int BiconeX(object O, float x, float y, float z)
{
	box b = bounds(O);
	return fabsf(U(x, b.xMin, b.xMax))+sqrt(sq(U(y, b.yMin, b.yMax))+sq(U(z, b.zMin, b.zMax))) < 1;
}

int BiconeY(object O, float x, float y, float z)
{
	box b = bounds(O);
	return fabsf(U(y, b.yMin, b.yMax))+sqrt(sq(U(z, b.zMin, b.zMax))+sq(U(x, b.xMin, b.xMax))) < 1;
}

int BiconeZ(object O, float x, float y, float z)
{
	box b = bounds(O);
	return fabsf(U(z, b.zMin, b.zMax))+sqrt(sq(U(x, b.xMin, b.xMax))+sq(U(y, b.yMin, b.yMax))) < 1;
}

/* elliptic rods, reference src/shapes.c:53-69 */
int RodX(object O, float x, float y, float z)
{
	box b = bounds(O);
	return IN(x, b.xMin, b.xMax) && sq(U(y, b.yMin, b.yMax))+sq(U(z, b.zMin, b.zMax)) < 1;
}

int RodY(object O, float x, float y, float z)
{
	box b = bounds(O);
	return IN(y, b.yMin, b.yMax) && sq(U(x, b.xMin, b.xMax))+sq(U(z, b.zMin, b.zMax)) < 1;
}

int RodZ(object O, float x, float y, float z)
{
	box b = bounds(O);
	return IN(z, b.zMin, b.zMax) && sq(U(x, b.xMin, b.xMax))+sq(U(y, b.yMin, b.yMax)) < 1;
}

/* rhombic rods, reference src/shapes.c:71-87 */
int DRodX(object O, float x, float y, float z)
{
	box b = bounds(O);
	return IN(x, b.xMin, b.xMax) && fabsf(U(y, b.yMin, b.yMax))+fabsf(U(z, b.zMin, b.zMax)) <= 1;
}

int DRodY(object O, float x, float y, float z)
{
	box b = bounds(O);
	return IN(y, b.yMin, b.yMax) && fabsf(U(z, b.zMin, b.zMax))+fabsf(U(x, b.xMin, b.xMax)) <= 1;
}

int DRodZ(object O, float x, float y, float z)
{
	box b = bounds(O);
	return IN(z, b.zMin, b.zMax) && fabsf(U(x, b.xMin, b.xMax))+fabsf(U(y, b.yMin, b.yMax)) <= 1;
}

/* hexagonal rods: axis first letter, flat sides normal to the second
 * (reference src/shapes.c:89-123) */
int HRodXY(object O, float x, float y, float z)
{
	box b = bounds(O);
	return IN(x, b.xMin, b.xMax) && INOPEN(z, b.zMin, b.zMax) && fabsf(U(z, b.zMin, b.zMax))+fabsf(U(y, b.yMin, b.yMax))*2 < 2;
}

int HRodYZ(object O, float x, float y, float z)
{
	box b = bounds(O);
	return IN(y, b.yMin, b.yMax) && INOPEN(x, b.xMin, b.xMax) && fabsf(U(x, b.xMin, b.xMax))+fabsf(U(z, b.zMin, b.zMax))*2 < 2;
}

int HRodZX(object O, float x, float y, float z)
{
	box b = bounds(O);
	return IN(z, b.zMin, b.zMax) && INOPEN(y, b.yMin, b.yMax) && fabsf(U(y, b.yMin, b.yMax))+fabsf(U(x, b.xMin, b.xMax))*2 < 2;
}

int HRodXZ(object O, float x, float y, float z)
{
	box b = bounds(O);
	return IN(x, b.xMin, b.xMax) && INOPEN(y, b.yMin, b.yMax) && fabsf(U(y, b.yMin, b.yMax))+fabsf(U(z, b.zMin, b.zMax))*2 < 2;
}

int HRodYX(object O, float x, float y, float z)
{
	box b = bounds(O);
	return IN(y, b.yMin, b.yMax) && INOPEN(z, b.zMin, b.zMax) && fabsf(U(z, b.zMin, b.zMax))+fabsf(U(x, b.xMin, b.xMax))*2 < 2;
}

int HRodZY(object O, float x, float y, float z)
{
	box b = bounds(O);
	return IN(z, b.zMin, b.zMax) && INOPEN(x, b.xMin, b.xMax) && fabsf(U(x, b.xMin, b.xMax))+fabsf(U(y, b.yMin, b.yMax))*2 < 2;
}


/* --- compound shapes (reference src/shapes.c:128-221) --- */

/* shift by f[0] (reference src/shapes.c:128-131) */
int Translation(object O, float x, float y, float z)
{
	object *o = O.p;
	return o->S(*o, x-O.f[0][0], y-O.f[0][1], z-O.f[0][2]);
}

/* rotation by angles f[0] (degrees) about centre f[1]; the trigonometric
 * values are single-precision glibc results of the degree angle
 * converted in double (reference src/shapes.c:133-140) */
int Rotation(object O, float x, float y, float z)
{
	object *o = O.p;
	x -= O.f[1][0], y -= O.f[1][1], z -= O.f[1][2];
	float cx = cosf(O.f[0][0]*PI/180.), sx = sinf(O.f[0][0]*PI/180.);
	float cy = cosf(O.f[0][1]*PI/180.), sy = sinf(O.f[0][1]*PI/180.);
	float cz = cosf(O.f[0][2]*PI/180.), sz = sinf(O.f[0][2]*PI/180.);
	float u = cz*x+sz*y, v = cz*y-sz*x;
	return o->S(*o, cy*u-sy*z, cx*v+sx*(cy*z+sy*u), cx*(cy*z+sy*u)-sx*v);
}

/* union / intersection / difference over f[0][0] members
 * (reference src/shapes.c:142-159) */
int Combination(object O, float x, float y, float z)
{
	object *o = O.p;
	int N = O.f[0][0];
	for (int n = 0; n < N; n++) if (o[n].S(o[n], x, y, z)) return 1;
	return 0;
}

int Intersection(object O, float x, float y, float z)
{
	object *o = O.p;
	int N = O.f[0][0];
	for (int n = 0; n < N; n++) if (!o[n].S(o[n], x, y, z)) return 0;
	return 1;
}

int Difference(object O, float x, float y, float z)
{
	object *o = O.p;
	int N = O.f[0][0];
	if (!o[0].S(o[0], x, y, z)) return 0;
	for (int n = 1; n < N; n++) if (o[n].S(o[n], x, y, z)) return 0;
	return 1;
}

/* fold one coordinate into the unit cell of a lattice with pitch a and
 * count c (c <= 0: infinite); arithmetic in double as in the reference
 * (src/shapes.c:164-178) */
static float foldAxis(float v, float a, float c, float lo, float hi)
{
	if (c) v += 0.5 * (c-1) * a;
	float q = floor((v + 0.5 * (a - lo - hi)) / a);
	v -= a * (c > 0 ? MAX(0, MIN(q, c-1)) : q);
	return v;
}

/* reference src/shapes.c:161-181 */
int Lattice(object O, float x, float y, float z)
{
	object *o = O.p;
	if (O.f[0][0]) x = foldAxis(x, O.f[0][0], O.f[0][1], o->f[0][0], o->f[0][1]);
	if (O.f[1][0]) y = foldAxis(y, O.f[1][0], O.f[1][1], o->f[1][0], o->f[1][1]);
	if (O.f[2][0]) z = foldAxis(z, O.f[2][0], O.f[2][1], o->f[2][0], o->f[2][1]);
	return o->S(*o, x, y, z) ? 1 : 0;
}

/* lattice plus the lattice shifted by half a period (one fewer cell)
 * (reference src/shapes.c:183-191) */
int DLattice(object O, float x, float y, float z)
{
	if (Lattice(O, x, y, z)) return 1;
	for (int d = 0; d < 3; d++) if (O.f[d][0]) O.f[d][1] -= O.f[d][1] ? 1 : 2;
	return Lattice(O, x, y, z) ? 1 : 0;
}

/* N-fold rotational copies about an axis through f[1]
 * (reference src/shapes.c:193-221) */
int CLatticeX(object O, float x, float y, float z)
{
	object *o = O.p;
	float y0 = O.f[1][0], z0 = O.f[1][1];
	int N = O.f[0][0];
	for (int n = 0; n < N; n++) {
		float t = 2 * PI * n / N;
		if (o->S(*o, x, (y-y0)*cosf(t) + (z-z0)*sinf(t) + y0, (z-z0)*cosf(t) - (y-y0)*sinf(t) + z0)) return 1;
	}
	return 0;
}

int CLatticeY(object O, float x, float y, float z)
{
	object *o = O.p;
	float x0 = O.f[1][0], z0 = O.f[1][1];
	int N = O.f[0][0];
	for (int n = 0; n < N; n++) {
		float t = 2 * PI * n / N;
		if (o->S(*o, (x-x0)*cosf(t) + (z-z0)*sinf(t) + x0, y, (z-z0)*cosf(t) - (x-x0)*sinf(t) + z0)) return 1;
	}
	return 0;
}

int CLatticeZ(object O, float x, float y, float z)
{
	object *o = O.p;
	float x0 = O.f[1][0], y0 = O.f[1][1];
	int N = O.f[0][0];
	for (int n = 0; n < N; n++) {
		float t = 2 * PI * n / N;
		if (o->S(*o, (x-x0)*cosf(t) + (y-y0)*sinf(t) + x0, (y-y0)*cosf(t) - (x-x0)*sinf(t) + y0, z)) return 1;
	}
	return 0;
}

/* height-map membership over a float** grid in O.p
 * (reference src/shapes.c:226-235) */
int ImportContour(object O, float x, float y, float z)
{
	float **f = O.p;
	if (O.f[0][0] < x && x < O.f[0][1] && O.f[1][0] < y && y < O.f[1][1]) {
		int i = O.f[0][2] * (x - O.f[0][0]) / (O.f[0][1] - O.f[0][0]);
		int j = O.f[1][2] * (y - O.f[1][0]) / (O.f[1][1] - O.f[1][0]);
		if (O.f[2][0] <= f[i][j] && f[i][j] <= O.f[2][1]) return 1;
	}
	return 0;
}
