/*
 * input.h -- project replacement for the reference's compile-time input
 * (reference: input.h:45-102).  Used ONLY when the reference C sources are
 * compiled in place into oracle/_ref/ by oracle/build_ref.py; it is test
 * infrastructure, never part of the product.
 *
 * The reference fixes the grid and physics knobs with #defines.  Here the grid
 * size comes from -DREF_NR/-DREF_NPHI/-DREF_NZ (one shared object per grid
 * size, because the reference's arrays are static), and every physics knob the
 * reference reads as a plain identifier is a global double so the harness can
 * set it at run time.  Arithmetic on a global double is bit-identical to the
 * same arithmetic on the literal the reference's #define would have expanded
 * to.
 *
 * Grid: the uniform cylindrical disc grid r in [0.1,1.5], phi in [0,2pi),
 * z in [-0.5,0.5]; with -DREF_SHIPPED the reference's own stretched grid at
 * the given size (its input.h uses 240x64x200).  The reference builds the grid with x[0]=x0-dx0 and
 * x[i+1]=x[i]+dx[i] (cylindricalgrid.h:36-47), so the first interior centre is
 * x0; stretching is disabled by putting lx/lz beyond the domain.
 */

#ifndef REF_NR
#error "REF_NR/REF_NPHI/REF_NZ must be given on the command line"
#endif

#define ix REF_NR
#define jy REF_NPHI
#define kz REF_NZ

#ifdef REF_SHIPPED
/* the reference's own stretched grid (input.h:48-72): uniform dx0 up to
 * r = lx and dz0 up to z = lz, then cells growing by stretchratio to at most
 * 50 dx0 / 50 dz0; z starts at the midplane */
#define lx 2.0
#define ly pi2
#define lz 0.03
#define dx0 0.01
#define dz0 0.0003
#define x0 0.04
#define y0 0.0
#define z0 0.0
#else
#define lx 1.0e30
#define ly pi2
#define lz 1.0e30
#define dx0 (1.4/(double)REF_NR)
#define dz0 (1.0/(double)REF_NZ)
#define x0 (0.1+0.5*dx0)
#define y0 0.0
#define z0 (-0.5+0.5*dz0)
#endif
#define stretchratio 1.05
#define rin 0.1

#define margin 2

#define ixmax (ix+margin)
#define jymax (jy+margin)
#define kzmax (kz+margin)
#define ixmax1 (ixmax-1)
#define jymax1 (jymax-1)
#define kzmax1 (kzmax-1)

#define dy0 (ly/(double)jy)

#define irin ((int)(rin/dx0))

double dxmax=50.0*dx0;
double dzmax=50.0*dz0;

/* run-time knobs (the reference has these as #defines, input.h:58-84) */
double cfl=0.4;
double dtmin=1.0e-9;
double rhocr=1.0e-4;
double prcr=1.0e-3;
double betacr=0.1;
#define oneobetacr (1.0/betacr)
#define nstop 10000000
#define tint 0.05
#define tstop 40.0

double tout=tint;

double epssp0=0.05;
double tausp=200.0*1.0e+6*year/t0;
double scalez=0.03;
double scaler=0.7;
double scalephase=0.1;
int armnum=2;
double omegasp=10.0e+5/omega0*oneokpc;
double omegapattern=10.0e+5/omega0*oneokpc;
double pitch=15.0*M_PI/180.0;

int restartsw=0;
int nout=0;
