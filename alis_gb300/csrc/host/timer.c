/*
 * timer.c -- the loop timer, the public ghost-copy helper and the
 * nonlinear coupling entry points.
 */
#include <sys/time.h>
#include "engine.h"

/* Progress line "[elapsed/estimated] [n/N: %]" at most once a second;
 * returns n <= N, which is the loop condition of every ALiS program
 * (reference src/update.c:14-45).  When it ends a loop it also flushes
 * and syncs every backend buffer, so that host reads after the loop
 * (phaser arrays, fields) see final values. */
int (timer)(long int n, long int N, char *str, ...)
{
	static long int first, prev;
	static unsigned long long t0, tPrev;
	struct timeval now;
	gettimeofday(&now, 0);
	unsigned long long t = now.tv_sec * 1000000ULL + now.tv_usec;
	if (!n || !first) {
		first = prev = n;
		t0 = tPrev = t;
	} else if (n > N || t/1000000ULL > tPrev/1000000ULL) {
		unsigned long long el = t - t0;
		unsigned long long est = el + (N-n+1) * (t-tPrev) / (n-prev);
		if (est - el > 3600000000ULL) est -= est % 60000000ULL;
		prev = n;
		tPrev = t;
		if (str[0]) printf("\r%s ", str);
		else printf("\r");
		printf("[%02llu:%02llu:%02llu/%02llu:%02llu:%02llu] [%ld/%ld: %.1f%%]",
			el/3600000000ULL, el%3600000000ULL/60000000ULL, el%60000000ULL/1000000ULL,
			est/3600000000ULL, est%3600000000ULL/60000000ULL, est%60000000ULL/1000000ULL,
			(n-1), N, 100.0*(n-1)/N);
		fflush(stdout);
		if (n > N) printf("\n");
	}
	if (n > N) alis_be_sync_all();
	return n <= N;
}

/* Host copy of boundary ghost cells: F = cos F' + sin G', G = cos G' -
 * sin F' from the cells (i+iAlt, j+jAlt, k+kAlt) (reference
 * src/update.c:182-191).  Operates on host arrays; the time steps do the
 * same on the device. */
void (copyBoundary)(float ***F, float ***G, float cosk, float sink, int iMin, int iMax, int jMin, int jMax, int kMin, int kMax, int iAlt, int jAlt, int kAlt)
{
	if (G) {
		for (int i = iMin; i <= iMax; i++) for (int j = jMin; j <= jMax; j++) for (int k = kMin; k <= kMax; k++) {
			F[i][j][k] = cosk * F[i+iAlt][j+jAlt][k+kAlt] + sink * G[i+iAlt][j+jAlt][k+kAlt];
			G[i][j][k] = cosk * G[i+iAlt][j+jAlt][k+kAlt] - sink * F[i+iAlt][j+jAlt][k+kAlt];
		}
	} else {
		for (int i = iMin; i <= iMax; i++) for (int j = jMin; j <= jMax; j++) for (int k = kMin; k <= kMax; k++)
			F[i][j][k] = cosk * F[i+iAlt][j+jAlt][k+kAlt];
	}
}

/* chi(2) coupling between worlds (reference src/update.c:358-411) is not
 * part of the GPU engine; the entry points exist so programs link. */
/* second-harmonic generation and three-wave mixing (reference
 * src/update.c:386-411) */
void nonLinearSHG(world WS, world WP, float Alt)
{
	alis_be_nonlinear(WS, WP, WP, Alt);
}

void nonLinearTWM(world WS, world WP1, world WP2, float Alt)
{
	alis_be_nonlinear(WS, WP1, WP2, Alt);
}
