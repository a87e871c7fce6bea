/*
 * ref_harness.c -- drives the UNMODIFIED reference C sources (compiled in
 * place from the reference tree by oracle/build_ref.py) through a small
 * exported C API, so tests can run the reference's own step on a chosen state.
 *
 * Test infrastructure only: this file and its build output (oracle/_ref/) are
 * the checker, never the product.  Nothing here is shipped or timed as ours.
 *
 * What the harness adds around the reference (it changes none of its code):
 *   - prototypes the reference relies on implicitly: cot() (called in
 *     spiralgravity.h:39, never defined), Cooling() (setdt.h:54), Check()
 *     (halfstep.h:163);
 *   - run-time variant selection by redirecting the names the stage functions
 *     call (halfstep.h:40-77, firststep.h:37-78): minmod, MC, van Leer or
 *     superbee limiter, HLLD or HLL solver, and the source function
 *     (halfstep.h:84-86, firststep.h:85-89);
 *   - a cooling on/off switch in front of Cooling() (cooling.h:22);
 *   - TVD-RK3 driven exactly as the commented block of tvdrungekutta.h:21,63-83
 *     (psi factor exp(-dt*ch/cr/3), then FirstStep, SecondStep, ThirdStep);
 *   - the step loop body of main.c:319-351 (Setdt, dt guard, SpiralGravity,
 *     TVDRK, t+=dt) with the guard reported instead of exit(1).
 */
#define _GNU_SOURCE
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <time.h>
#include <sys/stat.h>
#include <omp.h>

double cot(double x);

#include "maxmin.h"
#include "constant.h"
#include "input.h"
#include "commonfield.h"
#include "commontemp.h"
#include "commongrid.h"

int Check(double dummyU[][ixmax][jymax][kzmax], double dummyV[][ixmax][jymax][kzmax]);
int ref_cooling_switch(double dummyrho, double dummypr);
int InitialGravity(void);

#define Cooling ref_cooling_switch
#include "cylindricalgrid.h"
#include "setdt.h"
#include "xboundary.h"
#include "yboundary.h"
#include "zboundary.h"
#include "centralboundary.h"
#include "xvlrboundary.h"
#include "yvlrboundary.h"
#include "zvlrboundary.h"
#include "vtou.h"
#include "utov.h"
#include "saveinitial.h"
#include "model.h"
#include "initialgravity.h"
#include "spiralgravity.h"
#undef Cooling
#include "cooling.h"
#define Cooling ref_cooling_switch
#include "source.h"
#include "vlrtoulr.h"
#include "vlrulrtoflr.h"
#include "vlrulrtoglr.h"
#include "vlrulrtohlr.h"
#include "primitivetof.h"
#include "primitivetog.h"
#include "primitivetoh.h"
#include "glmsourcesolver.h"
#include "limiterx.h"
#include "limitery.h"
#include "limiterz.h"
#include "hlldx.h"
#include "hlldy.h"
#include "hlldz.h"
#include "hllx.h"
#include "hlly.h"
#include "hllz.h"

/* ---- run-time variant selection ------------------------------------------ */
static int g_limiter = 0;   /* 0 minmod, 1 MC, 2 van Leer, 3 superbee */
static int g_solver = 0;    /* 0 HLLD, 1 HLL */
static int g_scheme = 3;    /* 2 = live RK2 (Halfstep/Fullstep), 3 = RK3 */
static int g_cooling = 0;   /* 0 off, 1 on */
static int g_gravity = 0;   /* 0 off, 1 spiral+axisymmetric on */
static int g_source = 0;    /* 0 SpiralGravityCooling, 1 AxiGravity(Cooling), 2 UniformGz, 3 NoSource */

static int dispatch_lim_x(void)
{
	return g_limiter == 3 ? SuperbeeLimiterX() : g_limiter == 2 ? VanLeerLimiterX()
	     : g_limiter ? MCLimiterX() : MinmodLimiterX();
}
static int dispatch_lim_y(void)
{
	return g_limiter == 3 ? SuperbeeLimiterY() : g_limiter == 2 ? VanLeerLimiterY()
	     : g_limiter ? MCLimiterY() : MinmodLimiterY();
}
static int dispatch_lim_z(void)
{
	return g_limiter == 3 ? SuperbeeLimiterZ() : g_limiter == 2 ? VanLeerLimiterZ()
	     : g_limiter ? MCLimiterZ() : MinmodLimiterZ();
}
static int dispatch_rs_x(void) { return g_solver ? HLLX() : HLLDX(); }
static int dispatch_rs_y(void) { return g_solver ? HLLY() : HLLDY(); }
static int dispatch_rs_z(void) { return g_solver ? HLLZ() : HLLDZ(); }

static int dispatch_source(double dV[][ixmax][jymax][kzmax], double dS[][ixmax][jymax][kzmax])
{
	if (g_source == 1) return g_cooling ? AxiGravityCooling(dV, dS) : AxiGravity(dV, dS);
	if (g_source == 2) return UniformGz(dV, dS);
	if (g_source == 3) return NoSource(dV, dS);
	return SpiralGravityCooling(dV, dS);
}

#define SpiralGravityCooling dispatch_source
#define MinmodLimiterX dispatch_lim_x
#define MinmodLimiterY dispatch_lim_y
#define MinmodLimiterZ dispatch_lim_z
#define HLLDX dispatch_rs_x
#define HLLDY dispatch_rs_y
#define HLLDZ dispatch_rs_z
#include "halfstep.h"
#include "fullstep.h"
#include "firststep.h"
#include "secondstep.h"
#include "thirdstep.h"
#include "tvdrungekutta.h"
#undef SpiralGravityCooling
#undef MinmodLimiterX
#undef MinmodLimiterY
#undef MinmodLimiterZ
#undef HLLDX
#undef HLLDY
#undef HLLDZ
#include "check.h"
#include "output.h"
#include "restartread.h"
#undef Cooling

int ref_cooling_switch(double dummyrho, double dummypr)
{
	return g_cooling ? Cooling(dummyrho, dummypr) : 0;
}

double cot(double x) { return 1.0 / tan(x); }

/* ---- exported API --------------------------------------------------------- */

#define NCELL ((size_t)ixmax * jymax * kzmax)
#define NFACE ((size_t)ixmax1 * jymax1 * kzmax1)

void ref_dims(int *out)
{
	out[0] = ix; out[1] = jy; out[2] = kz;
	out[3] = ixmax; out[4] = jymax; out[5] = kzmax; out[6] = irin;
}

/* params: 0 cfl, 1 dtmin, 2 rhocr, 3 prcr, 4 betacr, 5 epssp0, 6 tausp,
 * 7 scalez, 8 scaler, 9 scalephase, 10 armnum, 11 omegasp, 12 omegapattern,
 * 13 pitch; flags: limiter, solver, scheme, cooling, gravity, source. */
void ref_set_params(const double *p, const int *flags)
{
	cfl = p[0]; dtmin = p[1]; rhocr = p[2]; prcr = p[3]; betacr = p[4];
	epssp0 = p[5]; tausp = p[6]; scalez = p[7]; scaler = p[8];
	scalephase = p[9]; armnum = (int)p[10]; omegasp = p[11];
	omegapattern = p[12]; pitch = p[13];
	g_limiter = flags[0]; g_solver = flags[1]; g_scheme = flags[2];
	g_cooling = flags[3]; g_gravity = flags[4]; g_source = flags[5];
}

void ref_grid(void) { CylindricalGrid(); }

/* back to the state of a fresh process: the reference keeps everything in
 * static arrays, which outlive one test case in a loaded library */
void ref_reset(void)
{
	memset(U, 0, sizeof U); memset(U1, 0, sizeof U1); memset(V, 0, sizeof V);
	memset(F, 0, sizeof F); memset(G, 0, sizeof G); memset(H, 0, sizeof H);
	memset(S, 0, sizeof S);
	memset(Grx, 0, sizeof Grx); memset(Gry, 0, sizeof Gry); memset(Grz, 0, sizeof Grz);
	memset(Grxaxi, 0, sizeof Grxaxi); memset(Gryaxi, 0, sizeof Gryaxi); memset(Grzaxi, 0, sizeof Grzaxi);
	memset(Vl, 0, sizeof Vl); memset(Vr, 0, sizeof Vr); memset(Ul, 0, sizeof Ul); memset(Ur, 0, sizeof Ur);
	memset(Fl, 0, sizeof Fl); memset(Fr, 0, sizeof Fr); memset(Gl, 0, sizeof Gl); memset(Gr, 0, sizeof Gr);
	memset(Hl, 0, sizeof Hl); memset(Hr, 0, sizeof Hr);
	memset(Uinitial, 0, sizeof Uinitial); memset(Vinitial, 0, sizeof Vinitial);
	memset(rhofloor, 0, sizeof rhofloor);
	dt = 0.0; ch = 0.0; t = 0.0; psicoef = 0.0;
}

/* the reference's Setdt() shares its running maximum between OpenMP threads
 * without a critical section (setdt.h:33,60-69): parity runs use one thread */
void ref_set_threads(int n) { omp_set_num_threads(n); }

/* 1D grid tables in the reference's order, each of the stated length. */
void ref_get_grid1d(double *xo, double *xmo, double *dxo, double *dxmo,
                    double *oneoxo, double *oneoxmo, double *oneodxo,
                    double *yo, double *zo, double *zmo, double *dzo,
                    double *dzmo, double *oneodzo, double *scalars)
{
	memcpy(xo, x, sizeof x); memcpy(xmo, xm, sizeof xm);
	memcpy(dxo, dx, sizeof dx); memcpy(dxmo, dxm, sizeof dxm);
	memcpy(oneoxo, oneox, sizeof oneox); memcpy(oneoxmo, oneoxm, sizeof oneoxm);
	memcpy(oneodxo, oneodx, sizeof oneodx);
	memcpy(yo, y, sizeof y); memcpy(zo, z, sizeof z); memcpy(zmo, zm, sizeof zm);
	memcpy(dzo, dz, sizeof dz); memcpy(dzmo, dzm, sizeof dzm);
	memcpy(oneodzo, oneodz, sizeof oneodz);
	scalars[0] = dy; scalars[1] = oneody; scalars[2] = minminlength;
	scalars[3] = oneominminlength;
}

/* 3D metric tables g1..g6 ([ixmax1][jymax1][kzmax1]) and minlength
 * ([ixmax][jymax][kzmax]); absorbing factors x(11), z(11), c((irin+1)*kzmax). */
void ref_get_metric(double *gout, double *minlen, double *xabs, double *zabs,
                    double *cabs, int *krin_out)
{
	memcpy(gout + 0 * NFACE, g1, sizeof g1); memcpy(gout + 1 * NFACE, g2, sizeof g2);
	memcpy(gout + 2 * NFACE, g3, sizeof g3); memcpy(gout + 3 * NFACE, g4, sizeof g4);
	memcpy(gout + 4 * NFACE, g5, sizeof g5); memcpy(gout + 5 * NFACE, g6, sizeof g6);
	memcpy(minlen, minlength, sizeof minlength);
	memcpy(xabs, x_absorb_factor, sizeof x_absorb_factor);
	memcpy(zabs, z_absorb_factor, sizeof z_absorb_factor);
	memcpy(cabs, c_absorb_factor, sizeof c_absorb_factor);
	memcpy(krin_out, krin, sizeof krin);
}

void ref_initial_gravity(void) { InitialGravity(); }

void ref_get_gravity(double *axi, double *gr)
{
	memcpy(axi + 0 * NCELL, Grxaxi, sizeof Grxaxi);
	memcpy(axi + 1 * NCELL, Gryaxi, sizeof Gryaxi);
	memcpy(axi + 2 * NCELL, Grzaxi, sizeof Grzaxi);
	memcpy(gr + 0 * NCELL, Grx, sizeof Grx);
	memcpy(gr + 1 * NCELL, Gry, sizeof Gry);
	memcpy(gr + 2 * NCELL, Grz, sizeof Grz);
}

void ref_set_gravity_axi(const double *axi)
{
	memcpy(Grxaxi, axi + 0 * NCELL, sizeof Grxaxi);
	memcpy(Gryaxi, axi + 1 * NCELL, sizeof Gryaxi);
	memcpy(Grzaxi, axi + 2 * NCELL, sizeof Grzaxi);
}

void ref_load(const double *Uin, const double *Vin, const double *Uinit,
              const double *Vinit, const double *rhof)
{
	memcpy(U, Uin, sizeof U); memcpy(V, Vin, sizeof V);
	memcpy(Uinitial, Uinit, sizeof Uinitial);
	memcpy(Vinitial, Vinit, sizeof Vinitial);
	memcpy(rhofloor, rhof, sizeof rhofloor);
}

void ref_store(double *Uout, double *Vout, double *U1out)
{
	if (Uout) memcpy(Uout, U, sizeof U);
	if (Vout) memcpy(Vout, V, sizeof V);
	if (U1out) memcpy(U1out, U1, sizeof U1);
}

/* the reference's own initial models, for the shipped production case */
void ref_galactic_disc3(void) { GalacticDisc3(); }
void ref_vtou(void) { VtoU(); }
void ref_save_initial(void) { SaveInitial(); }
void ref_get_initial(double *Uinit, double *Vinit, double *rhof)
{
	memcpy(Uinit, Uinitial, sizeof Uinitial);
	memcpy(Vinit, Vinitial, sizeof Vinitial);
	memcpy(rhof, rhofloor, sizeof rhofloor);
}

void ref_setdt(double *dt_out, double *ch_out)
{
	Setdt();
	*dt_out = dt; *ch_out = ch;
}

void ref_spiral_gravity(double tnow)
{
	t = tnow;
	SpiralGravity();
}

static void tvdrk3(void)
{
	psicoef = exp(-dt * ch * oneocr * oneo3);
	FirstStep();
	SecondStep();
	ThirdStep();
}

/* One step of main.c:319-351.  Returns 0, or 1 when the dt guard of
 * main.c:331 fires (the state is then left as Setdt found it). */
int ref_step(double *t_io, double *dt_out, double *ch_out, int *counters)
{
	t = *t_io;
	Setdt();
	*dt_out = dt; *ch_out = ch;
	if (isinf(dt) || dt < dtmin) return 1;
	if (g_gravity) SpiralGravity();
	if (g_scheme == 2) TVDRK(); else tvdrk3();
	counters[0] = rhoflag; counters[1] = prflag; counters[2] = oneobetaflag;
	t += dt;
	*t_io = t;
	return 0;
}

/* per-kernel probes: one direction's limiter and Riemann flux on the current V
 * with the given dt, ch (the values the stage functions read as globals). */
void ref_set_dtch(double dt_in, double ch_in, double psicoef_in)
{
	dt = dt_in; ch = ch_in; psicoef = psicoef_in;
}

void ref_limiter(int dir, double *Vlo, double *Vro)
{
	memset(Vl, 0, sizeof Vl); memset(Vr, 0, sizeof Vr);
	if (dir == 0) dispatch_lim_x(); else if (dir == 1) dispatch_lim_y(); else dispatch_lim_z();
	memcpy(Vlo, Vl, sizeof Vl); memcpy(Vro, Vr, sizeof Vr);
}

void ref_flux(int dir, double *Fo)
{
	if (dir == 0) { memset(F, 0, sizeof F); dispatch_lim_x(); dispatch_rs_x(); memcpy(Fo, F, sizeof F); }
	else if (dir == 1) { memset(G, 0, sizeof G); dispatch_lim_y(); dispatch_rs_y(); memcpy(Fo, G, sizeof G); }
	else { memset(H, 0, sizeof H); dispatch_lim_z(); dispatch_rs_z(); memcpy(Fo, H, sizeof H); }
}

void ref_source(double *So)
{
	SpiralGravityCooling(V, S);
	memcpy(So, S, sizeof S);
}

void ref_utov_check(double *Uio, double *Vo, int *counters)
{
	memcpy(U, Uio, sizeof U);
	UtoV(U, V);
	Check(U, V);
	memcpy(Uio, U, sizeof U); memcpy(Vo, V, sizeof V);
	counters[0] = rhoflag; counters[1] = prflag; counters[2] = oneobetaflag;
}

int ref_cooling(double rho, double pr) { return Cooling(rho, pr); }

/* BinaryOutput (output.h:1202) into directory ./<num> under cwd */
void ref_binary_output(int num, double tnow)
{
	nout = num; t = tnow;
	BinaryOutput();
}

/* GNUOutputCylinder() and GDLOutputCylinder() (output.h:25-390) into the
 * working directory */
void ref_text_output(int num, int step, double tnow)
{
	nout = num; nstep = step; t = tnow;
	GNUOutputCylinder();
	GDLOutputCylinder();
}

/* RestartRead(num) (restartread.h:9-143): V from ./<num>/, VtoU, Check */
void ref_restart_read(int num) { RestartRead(num); }

/* floor counters of the last Check() */
void ref_check_flags(int *out)
{
	out[0] = rhoflag; out[1] = prflag; out[2] = oneobetaflag;
}
