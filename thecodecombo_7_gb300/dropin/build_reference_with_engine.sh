#!/bin/sh
# Links the reference program (its own unmodified sources, where they lie)
# against the GPU engine, in the two forms fe_dropin.c supports: every file of
# the makefile's SRCS except the ones the drop-in replaces, plus fe_dropin.c,
# the project's FFTW3 shim (FFTW3 is not installed) and libfe.so.
#   MD form, flags -DNLIST -DEWALD -DSPME -DSTYPE  -> _build/md/spidey_gpu
#   MC form, flags -DNLIST -DEWALD -DMC -DSTYPE    -> _build/mc/spidey_gpu
# Output under thecodecombo_7_gb300/dropin/_build (git-ignored).
set -e
REF=${REF_DIR:?set REF_DIR to the reference source tree}
HERE=$(cd "$(dirname "$0")" && pwd)
PKG=$(dirname "$HERE")
ROOT=$(dirname "$PKG")
if [ ! -f "$REF/makefile" ]; then
  echo "reference sources not present; skipped"
  exit 0
fi
SRCS=$(sed -n '/^SRCS *=/,/^$/p' "$REF/makefile" | tr '\\\t' '  ' | sed 's/SRCS *=//' | tr -s ' ' '\n' | grep '\.c$')
CUDA=${CUDA_HOME:-/usr/local/cuda}
link() {
  form=$1; flags=$2; replaced=$3
  OUT="$HERE/_build/$form"
  mkdir -p "$OUT"
  FLAGS="-std=gnu99 -O2 -w $flags"
  objs=""
  for s in $SRCS; do
    case " $replaced " in *" $s "*) continue ;; esac
    o="$OUT/${s%.c}.o"
    gcc $FLAGS -I"$ROOT/oracle/fftw_shim" -I"$REF" -c "$REF/$s" -o "$o"
    objs="$objs $o"
  done
  gcc $FLAGS -I"$ROOT/oracle/fftw_shim" -I"$REF" -I"$ROOT/include" -c "$HERE/fe_dropin.c" \
      -o "$OUT/fe_dropin.o"
  gcc -std=gnu99 -O2 -c "$ROOT/oracle/fftw_shim/fftw_shim.c" -o "$OUT/fftw_shim.o"
  gcc -std=gnu99 -O2 -c "$ROOT/oracle/fe_fft.c" -o "$OUT/fe_fft.o"
  gcc -o "$OUT/spidey_gpu" $objs "$OUT/fe_dropin.o" "$OUT/fftw_shim.o" "$OUT/fe_fft.o" \
      -L"$PKG" -lfe -L"$CUDA/lib64" -lcudart -lcufft -Wl,-rpath,"$PKG" \
      -Wl,-rpath,"$CUDA/lib64" -lm
  echo "linked $OUT/spidey_gpu"
}
link md "-DNLIST -DEWALD -DSPME -DSTYPE" \
  "nblist.c cnonbond_nblist.c pme_qgrid.c pme_calc.c pme_setup.c pme_spline.c integrate_vverlet.c integrate_nhc.c pbc_all.c kinet.c forces.c drift.c isokin.c swap_box.c integrate_mts.c integrate_mts_nhc.c force_short.c force_long.c"
link mc "-DNLIST -DEWALD -DMC -DSTYPE" \
  "forces_mc.c enbnd_mc.c ewald_mc.c nblist_pivot.c drift.c"
