#!/bin/sh
# Builds the REFERENCE's own hot-path routines, from the unmodified sources
# where they lie, into oracle/_ref/ (git-ignored).  Used only to pin the
# oracle and to generate golden fixtures; the reference tree is only present
# on the development machine, so this is skipped elsewhere.
#
#   ref_harness       strict IEEE build (-O2 -ffp-contract=off, no fast-math):
#                     bit-reproducible, used for golden vectors
#   ref_harness_fast  the reference makefile's own flags (makefile:84-88:
#                     -O3 -ffast-math -funroll-all-loops -std=c99), for timing
#   ref_harness_dlist the strict build with -DDLIST (nl_check)
#   ref_harness_bgo   the strict build with -DBGO (the 12-10-6 pair form)
#   ref_harness_go    the Go-model routines of cgolik.c (-DGOLIK)
#
# Feature flags: -DNLIST -DEWALD -DSPME -DSTYPE.  FFTW3 is not installed, so
# the five FFTW symbols come from oracle/fftw_shim (the oracle's own FFT).
set -e
REF=${REF_DIR:?set REF_DIR to the reference source tree}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/defines.h" ]; then
  echo "build_ref: reference sources not present; skipped"
  exit 0
fi
mkdir -p "$OUT"
SRCS="nblist cnonbond_nblist pme_qgrid pme_spline pme_setup pme_calc forces
      cbond cbend curey ctorsion cimproper integrate_vverlet pbc_all kinet
      integrate_nhc setlj ewald drift integrate_mts integrate_mts_nhc force_short force_long"
FEAT="-DNLIST -DEWALD -DSPME -DSTYPE"
build() {
  name=$1; shift
  files=""
  for s in $SRCS; do files="$files $REF/$s.c"; done
  gcc "$@" $FEAT -I"$HERE/fftw_shim" -I"$REF" -w -o "$OUT/$name" \
      "$HERE/ref_harness.c" $files "$HERE/fftw_shim/fftw_shim.c" \
      "$HERE/fe_fft.c" -lm
}
build ref_harness -std=gnu99 -O2 -ffp-contract=off
build ref_harness_fast -std=c99 -D_POSIX_C_SOURCE=200809L -O3 -ffast-math -funroll-all-loops
# the DLIST build (nl_check and the list-time snapshot, nblist.c:583-647)
build ref_harness_dlist -std=gnu99 -O2 -ffp-contract=off -DDLIST
# the classic-Ewald Monte Carlo build (-DMC without SPME): enbnd_mc,
# ewald_kspace_mc and ewald_rspace_mc (ewald_mc.c:42-641), strict IEEE
gcc -std=gnu99 -O2 -ffp-contract=off -DNLIST -DEWALD -DMC -DSTYPE -I"$REF" -w \
    -o "$OUT/ref_harness_mc" "$HERE/ref_harness.c" \
    "$REF/nblist.c" "$REF/setlj.c" "$REF/ewald.c" "$REF/ewald_mc.c" "$REF/cplx.c" \
    "$REF/enbnd_mc.c" -lm
# the Brooks Go model's pair form (-DBGO: cnonbond_nblist.c:294-307), strict;
# -fcommon: defines.h declares a global of that build without extern, as the
# compilers of the reference's time merged (common symbols)
build ref_harness_bgo -std=gnu99 -O2 -ffp-contract=off -fcommon -DBGO
# the reference's own Go model (-DGOLIK, no STYPE: cgolik.c reads the
# per-box pair table ljset[k].pot[a][b]), strict IEEE
gcc -std=gnu99 -O2 -ffp-contract=off -DGOLIK -DNLIST -I"$REF" -w \
    -o "$OUT/ref_harness_go" "$HERE/ref_harness_go.c" "$REF/cgolik.c" -lm
echo "build_ref: built $OUT/ref_harness, $OUT/ref_harness_fast, $OUT/ref_harness_dlist, $OUT/ref_harness_mc, $OUT/ref_harness_bgo and $OUT/ref_harness_go"
