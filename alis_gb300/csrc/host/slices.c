/*
 * slices.c -- 1-D / 2-D cuts of a field function: snapshots, time
 * averages and single-frequency DFTs written as text or PNG images.
 *
 * Visualisation side of the reference src/slices.c.  PNG files are
 * produced by a small encoder in this file (uncompressed deflate blocks),
 * so no libpng is needed; HDF5 output is not built.  Graded grids are
 * resampled to the uniform base spacing before writing, as in the
 * reference's bilinear interpolation.
 */
#include <sys/stat.h>
#include <string.h>
#include <limits.h>
#include <stdint.h>
#include "engine.h"

/* --- graded-grid resampling (reference src/slices.c:25-64) ---
 * A slice of a graded grid is written on the uniform base grid: along
 * each axis the slice spans (index range [lo, hi] of the graded grid ->
 * range [LO, HI] of base-grid points), every base point n between graded
 * cells c and c + 1 gets the linear interpolation of the two.  Axes are
 * done in the order i, j, k; an axis done spans its base range in the
 * passes after it.  The arithmetic is the reference's: float positions,
 * float weights, one division per point. */

static float gridPos(world W, int axis, int c)
{
	return axis == 0 ? W->itox(W, c) : axis == 1 ? W->jtoy(W, c) : W->ktoz(W, c);
}

static float gridStep(world W, int axis)
{
	return axis == 0 ? W->dx : axis == 1 ? W->dy : W->dz;
}

static float ***resample(world W, slice S, float ***F)
{
	const int lo[3] = { S->iMin, S->jMin, S->kMin }, hi[3] = { S->iMax, S->jMax, S->kMax };
	const int LO[3] = { S->iMIN, S->jMIN, S->kMIN }, HI[3] = { S->iMAX, S->jMAX, S->kMAX };
	int from[3], to[3];             /* the current extent of the data per axis */
	for (int a = 0; a < 3; a++) from[a] = lo[a], to[a] = hi[a];
	float ***src = makeField(S->iMIN, S->iMAX, S->jMIN, S->jMAX, S->kMIN, S->kMAX), ***dst = F;
	for (int a = 0; a < 3; a++) {
		if (lo[a] == LO[a] && hi[a] == HI[a]) continue;
		float ***t = src; src = dst; dst = t;
		const int b = (a + 1) % 3, c = (a + 2) % 3;
		const float d = gridStep(W, a);
		for (int g = lo[a]; g < hi[a]; g++) {
			const float p0 = gridPos(W, a, g), p1 = gridPos(W, a, g+1);
			const int n0 = p0/d+(g>0?1:0), n1 = p1/d-(g<0?1:0);
			int at[3], next[3];
			for (at[b] = from[b]; at[b] <= to[b]; at[b]++) for (at[c] = from[c]; at[c] <= to[c]; at[c]++) {
				at[a] = g;
				next[0] = at[0], next[1] = at[1], next[2] = at[2], next[a] = g+1;
				const float v0 = src[at[0]][at[1]][at[2]], v1 = src[next[0]][next[1]][next[2]];
				for (int n = n0; n <= n1; n++) {
					at[a] = n;
					dst[at[0]][at[1]][at[2]] = (v0 * (p1 - n*d) + v1 * (n*d - p0)) / (p1 - p0);
				}
			}
		}
		from[a] = LO[a], to[a] = HI[a];
	}
	removeField(src, S->iMIN, S->jMIN, S->kMIN);
	return dst;
}

/* Index range of a slice along one axis: the box's ends as grid indices,
 * clipped to the grid (to the mirror image of the grid below a symmetry
 * plane), and the base-grid range the slice covers when it is resampled
 * (reference src/slices.c:67-97). */
static void sliceAxis(world W, int axis, float pMin, float pMax, int resampled, int r[4])
{
	const int MIN_[3] = { W->iMIN, W->jMIN, W->kMIN }, MAX_[3] = { W->iMAX, W->jMAX, W->kMAX };
	const int sym = (axis == 0 ? W->xMinSur : axis == 1 ? W->yMinSur : W->zMinSur) == SYM;
	int a = axis == 0 ? W->xtoi(W, pMin) : axis == 1 ? W->ytoj(W, pMin) : W->ztok(W, pMin);
	int b = axis == 0 ? W->xtoi(W, pMax) : axis == 1 ? W->ytoj(W, pMax) : W->ztok(W, pMax);
	if (b > MAX_[axis]) b = MAX_[axis];
	const int floorIdx = sym ? -MAX_[axis] : MIN_[axis];
	if (a < floorIdx) a = floorIdx;
	r[0] = a, r[1] = b, r[2] = a, r[3] = b;
	if (a != b && resampled) {
		/* MIN / MAX of an index and a base-grid position, as float */
		const float d = gridStep(W, axis), ea = gridPos(W, axis, a)/d, eb = gridPos(W, axis, b)/d;
		r[2] = a < ea ? a : ea;
		r[3] = b > eb ? b : eb;
	}
}

/* A slice through the given box.  2-D slices of a world with eps^-1 maps
 * carry the index contour of the objects, scaled to at most 0.5, for the
 * image writers to overlay (reference src/slices.c:98-117). */
slice createSlice(world W, float xMin, float xMax, float yMin, float yMax, float zMin, float zMax)
{
	slice S = calloc(1, sizeof *S);
	const int graded = W->Res.nug.x.m>1 || W->Res.nug.y.m>1 || W->Res.nug.z.m>1;
	if (graded) S->interpolate = resample;
	const float box[3][2] = { { xMin, xMax }, { yMin, yMax }, { zMin, zMax } };
	int r[3][4];
	for (int a = 0; a < 3; a++) sliceAxis(W, a, box[a][0], box[a][1], graded, r[a]);
	S->iMin = r[0][0], S->iMax = r[0][1], S->iMIN = r[0][2], S->iMAX = r[0][3];
	S->jMin = r[1][0], S->jMax = r[1][1], S->jMIN = r[1][2], S->jMAX = r[1][3];
	S->kMin = r[2][0], S->kMax = r[2][1], S->kMIN = r[2][2], S->kMAX = r[2][3];
	S->iNUM = 1-S->iMIN+S->iMAX;
	S->jNUM = 1-S->jMIN+S->jMAX;
	S->kNUM = 1-S->kMIN+S->kMAX;
	S->F = makeField(S->iMIN, S->iMAX, S->jMIN, S->jMAX, S->kMIN, S->kMAX);
	const int flat = S->iMin == S->iMax || S->jMin == S->jMax || S->kMin == S->kMax;
	if (!W->CE->x || !W->CE->y || !W->CE->z || !flat) return S;
	S->C = makeField(S->iMIN, S->iMAX, S->jMIN, S->jMAX, S->kMIN, S->kMAX);
	float top = 0;
	for (int i = S->iMIN; i <= S->iMAX; i++) for (int j = S->jMIN; j <= S->jMAX; j++) for (int k = S->kMIN; k <= S->kMAX; k++) {
		const float v = S->C[i][j][k] = ContourRI(W, i, j, k);
		if (top < v) top = v;
	}
	if (top) for (int i = S->iMIN; i <= S->iMAX; i++) for (int j = S->jMIN; j <= S->jMAX; j++) for (int k = S->kMIN; k <= S->kMAX; k++)
		S->C[i][j][k] = 0.5 * S->C[i][j][k] / top;
	return S;
}

void deleteSlice(slice S)
{
	if (S->F) removeField(S->F, S->iMIN, S->jMIN, S->kMIN);
	if (S->C) removeField(S->C, S->iMIN, S->jMIN, S->kMIN);
	free(S);
}


/* bring the host mirrors up to date over the slice (the whole world when
 * the backend cannot do it for the box) and hold further syncs of W while
 * the field functions are evaluated; returns whether syncs are held */
static int syncSlice(world W, slice S)
{
	int held = alis_be_sync_box(W, S->iMin, S->iMax, S->jMin, S->jMax, S->kMin, S->kMax);
	if (held) alis_be_hold_sync(W);
	else alis_be_sync_world(W);
	return held;
}

static void releaseSlice(int held)
{
	if (held) alis_be_hold_sync(0);
}


/* --- writers (reference src/slices.c:128-211) --- */

void (h5)(world W, slice S, float Max, char *F, char *filename, unsigned long int *cmap)
{
	(void)W; (void)S; (void)Max; (void)F; (void)filename; (void)cmap;
	fprintf(stderr, "alis: h5 slice output is unavailable (built without HDF5)\n");
	exit(1);
}

void (txt)(world W, slice S, float Max, char *F, char *filename, unsigned long int *cmap)
{
	(void)Max; (void)F; (void)cmap;
	int d = 0, dim[3] = {0};
	FILE *File = fopen(strcat(filename, ".txt"), "w");
	if (!File) return;
	if (S->iMin != S->iMax) dim[d++] = S->iNUM;
	if (S->jMin != S->jMax) dim[d++] = S->jNUM;
	if (S->kMin != S->kMax) dim[d++] = S->kNUM;
	if (d == 3) printf("Can't write 3D slice to txt file.\n"), exit(0);
	if (d == 1) {
		if (S->iMin != S->iMax) for (int i = S->iMin; i <= S->iMax; i++) fprintf(File, "%f\t%e\n", W->itox(W, i), S->F[i][S->jMin][S->kMin]);
		if (S->jMin != S->jMax) for (int j = S->jMin; j <= S->jMax; j++) fprintf(File, "%f\t%e\n", W->jtoy(W, j), S->F[S->iMin][j][S->kMin]);
		if (S->kMin != S->kMax) for (int k = S->kMin; k <= S->kMax; k++) fprintf(File, "%f\t%e\n", W->ktoz(W, k), S->F[S->iMin][S->jMin][k]);
	} else {
		if (S->interpolate) S->F = S->interpolate(W, S, S->F);
		float *base = &S->F[S->iMIN][S->jMIN][S->kMIN];
		for (int j = dim[1]-1; j >= 0; j--) {
			fprintf(File, "%e", base[j]);
			for (int i = 1; i < dim[0]; i++) fprintf(File, "\t%e", base[dim[1]*i+j]);
			fprintf(File, "\n");
		}
	}
	fclose(File);
}

/* minimal PNG: RGB8, one IDAT of stored (uncompressed) deflate blocks */
static uint32_t crcTable[256];
static void crcInit(void)
{
	for (uint32_t n = 0; n < 256; n++) {
		uint32_t c = n;
		for (int k = 0; k < 8; k++) c = c & 1 ? 0xEDB88320u ^ (c >> 1) : c >> 1;
		crcTable[n] = c;
	}
}
static uint32_t crc(uint32_t c, const unsigned char *b, size_t n)
{
	for (size_t q = 0; q < n; q++) c = crcTable[(c ^ b[q]) & 0xFF] ^ (c >> 8);
	return c;
}
static void put32(unsigned char *p, uint32_t v) { p[0] = v>>24, p[1] = v>>16, p[2] = v>>8, p[3] = v; }
static void chunk(FILE *f, const char *type, const unsigned char *data, size_t n)
{
	unsigned char h[8];
	put32(h, n);
	memcpy(h+4, type, 4);
	fwrite(h, 1, 8, f);
	if (n) fwrite(data, 1, n, f);
	uint32_t c = crc(0xFFFFFFFFu, (const unsigned char*)type, 4);
	c = crc(c, data, n) ^ 0xFFFFFFFFu;
	put32(h, c);
	fwrite(h, 1, 4, f);
}
static void writePNG(FILE *f, int w, int h, const unsigned char *rgb)
{
	static int init;
	if (!init) crcInit(), init = 1;
	size_t raw = (size_t)h*(1+3*w), blocks = (raw+65534)/65535;
	unsigned char *z = malloc(2 + raw + 5*blocks + 4), *p = z;
	uint32_t a = 1, b = 0;
	*p++ = 0x78, *p++ = 0x01;
	size_t left = raw, row = 0, col = 0;
	while (left) {
		size_t n = left < 65535 ? left : 65535;
		*p++ = left == n;
		*p++ = n & 0xFF, *p++ = n >> 8, *p++ = ~n & 0xFF, *p++ = (~n >> 8) & 0xFF;
		for (size_t q = 0; q < n; q++) {
			unsigned char v = col == 0 ? 0 : rgb[row*3*w + col-1];
			*p++ = v;
			a = (a + v) % 65521, b = (b + a) % 65521;
			if (++col == (size_t)(1+3*w)) col = 0, row++;
		}
		left -= n;
	}
	put32(p, (b << 16) | a), p += 4;
	unsigned char ihdr[13];
	put32(ihdr, w), put32(ihdr+4, h);
	ihdr[8] = 8, ihdr[9] = 2, ihdr[10] = ihdr[11] = ihdr[12] = 0;
	fwrite("\x89PNG\r\n\x1a\n", 1, 8, f);
	chunk(f, "IHDR", ihdr, 13);
	chunk(f, "IDAT", z, p - z);
	chunk(f, "IEND", 0, 0);
	free(z);
}

/* colour-mapped image of a 1-D (64 rows high) or 2-D slice with the index
 * contour overlay for field quantities (reference src/slices.c:167-211) */
void (png)(world W, slice S, float Max, char *F, char *filename, unsigned long int *cmap)
{
	int d = 0, dim[3] = {1, 1, 1};
	float Min = 0;
	if (cmap[0] > LONG_MAX) Min = -Max;
	if (F[0]=='L' && F[1]=='o' && F[2]=='g' && F[3]!='R' && F[4]!='I') Min = Max-3;
	if (S->iMin != S->iMax) dim[d++] = S->iNUM;
	if (S->jMin != S->jMax) dim[d++] = S->jNUM;
	if (S->kMin != S->kMax) dim[d++] = S->kNUM;
	if (d == 1) dim[2] = 64;
	if (d == 3) printf("Can't write 3D slice to png file.\n"), exit(0);
	FILE *File = fopen(strcat(filename, ".png"), "wb");
	if (!File) return;
	if (S->interpolate) S->F = S->interpolate(W, S, S->F);
	int stops = labs((long)cmap[0]);
	unsigned char *img = malloc((size_t)3*dim[0]*dim[1]*dim[2]);
	float *base = &S->F[S->iMIN][S->jMIN][S->kMIN];
	float *cb = S->C ? &S->C[S->iMIN][S->jMIN][S->kMIN] : 0;
	int plain = F[0]!='E' && F[0]!='H' && F[0]!='J' && F[0]!='U' && F[0]!='S' && F[0]!='i';
	for (int r = 0, j = dim[1]-1; j >= 0; j--) {
		unsigned char *row = img + (size_t)3*dim[0]*r;
		for (int i = 0; i < dim[0]; i++) {
			float C = !cb ? 1 : 1-cb[dim[1]*i+j];
			float f = (Max-Min) ? MAX(0, MIN(stops-1, (stops-1)*(base[dim[1]*i+j]-Min)/(Max-Min))) : 0;
			int n = f;
			if (plain) C = 1;
			if (n > stops-2) n = stops-2;
			for (int c = 0; c < 3; c++) {
				int sh = 16 - 8*c;
				row[3*i+c] = C * ((1-f+n) * (cmap[n+1]>>sh&0xFF) + (f-n) * (cmap[n+2]>>sh&0xFF));
			}
		}
		for (int q = 1; q < dim[2]; q++) memcpy(img + (size_t)3*dim[0]*(r+q), row, 3*dim[0]);
		r += dim[2];
	}
	writePNG(File, dim[0], dim[1]*dim[2], img);
	free(img);
	fclose(File);
}


/* --- per-call-site state (reference src/slices.c:214-239) --- */

typedef struct sliceq {
	world W;
	method M;
	char *name;
	float max, Max, ***F, ***G;
	long N;
	void *dev;                /* sliceFreqDom: the sums kept by the backend */
	struct sliceq *next;
} sliceq;

static sliceq *track(world W, char *ID, method M, sliceq **head)
{
	sliceq *q;
	for (q = *head; q; q = q->next) if (q->W == W && q->M == M && !strcmp(q->name, ID)) break;
	if (!q) {
		q = calloc(1, sizeof *q);
		q->W = W, q->M = M, q->name = strdup(ID);
		q->next = *head, *head = q;
		strcat(strcpy(ID, W->ID), q->name);
		if (q->name[0]=='/') mkdir(W->ID, 0755);
		if (ID[0] && ID[strlen(ID)-1]=='/') mkdir(ID, 0755);
	} else strcat(strcpy(ID, W->ID), q->name);
	q->N++;
	return q;
}

static int staticField(field F)
{
	return F==RI || F==LogRI || F==ContourRI || F==Contour || F==raweEffx || F==raweEffy || F==raweEffz || F==eEff;
}

/* replace the first '%' of a file name by "<field>-<slice>" */
static void expandName(char *filename, const char *f, const char *s)
{
	char rest[1024], *pct = strchr(filename, '%');
	if (!pct) return;
	strcpy(rest, pct+1);
	sprintf(pct, "%s-%s%s", f, s, rest);
}

void (sliceSnap)(world W, field F, slice S, char *f, char *s, ...)
{
	static sliceq *head;
	char *format, string[64], filename[1024];
	va_list ap;
	va_start(ap, s);
	int N = staticField(F) ? 0 : va_arg(ap, int);
	method M = va_arg(ap, method);
	unsigned long int *cmap = (M == png) ? va_arg(ap, unsigned long int *) : 0;
	float Max = (M == png) ? va_arg(ap, double) : 1;
	int step = (!N || N > (long)W->T) ? 1 : W->T/N;
	int skip = Max < 0 ? ((int)(-Max*W->T/step))*step : 0;
	format = va_arg(ap, char*);
	vsnprintf(filename, sizeof filename, format, ap);
	va_end(ap);
	expandName(filename, f, s);
	sliceq *q = track(W, filename, M, &head);
	if (N) sprintf(string, "%05ld", (q->N-skip)/step), strcat(filename, string);
	if (q->N % step) return;
	int held = syncSlice(W, S);
	float max = 0;
	for (int i = S->iMin; i <= S->iMax; i++) for (int j = S->jMin; j <= S->jMax; j++) for (int k = S->kMin; k <= S->kMax; k++)
		if (max < fabsf(S->F[i][j][k] = F(W, i, j, k))) max = fabsf(S->F[i][j][k]);
	releaseSlice(held);
	if (!Max) Max = max;
	else if (Max < 0) {
		Max = q->Max;
		if (q->max < max) q->max = max;
		if (q->N % skip == 0) q->Max = q->max, q->max = 0;
	}
	if (q->N > skip) M(W, S, Max ? Max : 1, f, filename, cmap);
}

void (sliceTimeAvg)(world W, field F, slice S, char *f, char *s, ...)
{
	static sliceq *head;
	char *format, string[64], filename[1024];
	va_list ap;
	va_start(ap, s);
	int N = staticField(F) ? 0 : va_arg(ap, int);
	method M = va_arg(ap, method);
	unsigned long int *cmap = (M == png) ? va_arg(ap, unsigned long int *) : 0;
	float Max = (M == png) ? va_arg(ap, double) : 1;
	format = va_arg(ap, char*);
	vsnprintf(filename, sizeof filename, format, ap);
	va_end(ap);
	expandName(filename, f, s);
	sliceq *q = track(W, filename, M, &head);
	if (N) sprintf(string, "%05ld", q->N / N), strcat(filename, string);
	if (q->N == 1) q->F = makeField(S->iMin, S->iMax, S->jMin, S->jMax, S->kMin, S->kMax);
	int held = syncSlice(W, S);
	for (int i = S->iMin; i <= S->iMax; i++) for (int j = S->jMin; j <= S->jMax; j++) for (int k = S->kMin; k <= S->kMax; k++)
		q->F[i][j][k] += F(W, i, j, k);
	releaseSlice(held);
	if (!N || q->N % N) return;
	float max = 0;
	for (int i = S->iMin; i <= S->iMax; i++) for (int j = S->jMin; j <= S->jMax; j++) for (int k = S->kMin; k <= S->kMax; k++)
		if (max < fabsf(S->F[i][j][k] = q->F[i][j][k] / N)) max = fabsf(S->F[i][j][k]);
	if (Max <= 0) Max = max;
	M(W, S, Max ? Max : 1, f, filename, cmap);
	for (int i = S->iMin; i <= S->iMax; i++) for (int j = S->jMin; j <= S->jMax; j++) for (int k = S->kMin; k <= S->kMax; k++)
		q->F[i][j][k] = 0;
}

void (sliceFreqDom)(world W, field F, slice S, char *f, char *s, int N, float L, ...)
{
	field *ok[30] = {Ex, Ey, Ez, Hx, Hy, Hz, iEx, iEy, iEz, iHx, iHy, iHz, rawEx, rawEy, rawEz, rawHx, rawHy, rawHz, Jx, Jy, Jz, rawJx, rawJy, rawJz, ScEx, ScEy, ScEz, SoEx, SoEy, SoEz};
	int n = 0;
	while (n < 30 && F != ok[n]) n++;
	if (n == 30) printf("\nThe %s field is not supported in sliceFreqDom().\n", f), exit(0);
	static sliceq *head;
	char *format, string[1100], filename[1024];
	va_list ap;
	va_start(ap, L);
	method M = va_arg(ap, method);
	unsigned long int *cmap = (M == png) ? va_arg(ap, unsigned long int *) : 0;
	float Max = (M == png) ? va_arg(ap, double) : 1;
	format = va_arg(ap, char*);
	vsnprintf(filename, sizeof filename, format, ap);
	va_end(ap);
	expandName(filename, f, s);
	sliceq *q = track(W, filename, M, &head);
	int box[6] = { S->iMin, S->iMax, S->jMin, S->jMax, S->kMin, S->kMax };
	float *F0 = 0, *G0 = 0;
	if (q->N == 1) {
		q->F = makeField(S->iMin, S->iMax, S->jMin, S->jMax, S->kMin, S->kMax);
		q->G = makeField(S->iMin, S->iMax, S->jMin, S->jMax, S->kMin, S->kMax);
		q->dev = alis_be_slice_dft_begin(W, box);
	}
	F0 = &q->F[S->iMin][S->jMin][S->kMin], G0 = &q->G[S->iMin][S->jMin][S->kMin];
	float re = cosf(2 * PI * q->N * W->dt / L);
	float im = sinf(2 * PI * q->N * W->dt / L);
	if (!(q->dev && alis_be_slice_dft_add(q->dev, W, F, re, im))) {
		/* a field function the backend does not evaluate: the sums so far come to the host */
		if (q->dev) alis_be_slice_dft_read(q->dev, F0, G0), alis_be_slice_dft_end(q->dev), q->dev = 0;
		int held = syncSlice(W, S);
		for (int i = S->iMin; i <= S->iMax; i++) for (int j = S->jMin; j <= S->jMax; j++) for (int k = S->kMin; k <= S->kMax; k++) {
			q->F[i][j][k] += F(W, i, j, k) * re;
			q->G[i][j][k] += F(W, i, j, k) * im;
		}
		releaseSlice(held);
	}
	if (q->N % N) return;
	if (q->dev) alis_be_slice_dft_read(q->dev, F0, G0);
	if (Max <= 0) {
		float max = 0;
		for (int i = S->iMin; i <= S->iMax; i++) for (int j = S->jMin; j <= S->jMax; j++) for (int k = S->kMin; k <= S->kMax; k++)
			if (max < sq(q->F[i][j][k])+sq(q->G[i][j][k])) max = sq(q->F[i][j][k])+sq(q->G[i][j][k]);
		if (Max < sqrtf(max) * 2 / q->N) Max = sqrtf(max) * 2 / q->N;
	}
	for (int p = 0; p < 12; p++) {
		for (int i = S->iMin; i <= S->iMax; i++) for (int j = S->jMin; j <= S->jMax; j++) for (int k = S->kMin; k <= S->kMax; k++)
			S->F[i][j][k] = (q->F[i][j][k] * cosf(p * PI / 6) + q->G[i][j][k] * sinf(p * PI / 6)) * 2 / q->N;
		snprintf(string, sizeof string, "%s%02d", filename, p+1);
		M(W, S, Max, f, string, cmap);
	}
}

float sliceMax(world W, field F, slice S)
{
	int held = syncSlice(W, S);
	float Max = 0, f;
	for (int i = S->iMin; i <= S->iMax; i++) for (int j = S->jMin; j <= S->jMax; j++) for (int k = S->kMin; k <= S->kMax; k++)
		if (Max < (f = fabsf(F(W, i, j, k)))) Max = f;
	releaseSlice(held);
	return Max;
}

static float sliceSumZ(world W, field F, slice S, int i, int j)
{
	float Sum = 0;
	for (int k = S->kMin+1; k < S->kMax; k++) Sum += W->CE->dz[k] * F(W, i, j, k);
	Sum += 0.5 * W->CE->dz[S->kMin] * F(W, i, j, S->kMin);
	Sum += 0.5 * W->CE->dz[S->kMax] * F(W, i, j, S->kMax);
	return Sum;
}

static float sliceSumY(world W, field F, slice S, int i)
{
	float Sum = 0;
	for (int j = S->jMin+1; j < S->jMax; j++) Sum += W->CE->dy[j] * sliceSumZ(W, F, S, i, j);
	Sum += 0.5 * W->CE->dy[S->jMin] * sliceSumZ(W, F, S, i, S->jMin);
	Sum += 0.5 * W->CE->dy[S->jMax] * sliceSumZ(W, F, S, i, S->jMax);
	return Sum;
}

float sliceSum(world W, field F, slice S)
{
	int held = syncSlice(W, S);
	float Sum = 0;
	for (int i = S->iMin+1; i < S->iMax; i++) Sum += W->CE->dx[i] * sliceSumY(W, F, S, i);
	Sum += 0.5 * W->CE->dx[S->iMin] * sliceSumY(W, F, S, S->iMin);
	Sum += 0.5 * W->CE->dx[S->iMax] * sliceSumY(W, F, S, S->iMax);
	releaseSlice(held);
	if (S->iMin==S->iMax) Sum /= W->CE->dx[S->iMin];
	if (S->jMin==S->jMax) Sum /= W->CE->dy[S->jMin];
	if (S->kMin==S->kMax) Sum /= W->CE->dz[S->kMin];
	return Sum;
}
