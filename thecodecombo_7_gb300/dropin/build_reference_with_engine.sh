#!/bin/sh
# Links the reference program (its own unmodified sources, where they lie)
# against the GPU engine: every file of the makefile's SRCS except the nine
# the drop-in replaces, plus fe_dropin.c, the project's FFTW3 shim (FFTW3 is
# not installed) and libfe.so.  Feature flags -DNLIST -DEWALD -DSPME -DSTYPE.
# Output: thecodecombo_7_gb300/dropin/_build/spidey_gpu (git-ignored).
set -e
REF=${REF:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
PKG=$(dirname "$HERE")
ROOT=$(dirname "$PKG")
OUT="$HERE/_build"
if [ ! -f "$REF/makefile" ]; then
  echo "reference sources not present; skipped"
  exit 0
fi
mkdir -p "$OUT"
REPLACED="nblist.c cnonbond_nblist.c pme_qgrid.c pme_calc.c integrate_vverlet.c integrate_nhc.c pbc_all.c kinet.c forces.c"
SRCS=$(sed -n '/^SRCS *=/,/^$/p' "$REF/makefile" | tr '\\\t' '  ' | sed 's/SRCS *=//' | tr -s ' ' '\n' | grep '\.c$')
FLAGS="-std=gnu99 -O2 -w -DNLIST -DEWALD -DSPME -DSTYPE"
objs=""
for s in $SRCS; do
  case " $REPLACED " in *" $s "*) continue ;; esac
  o="$OUT/${s%.c}.o"
  gcc $FLAGS -I"$ROOT/oracle/fftw_shim" -I"$REF" -c "$REF/$s" -o "$o"
  objs="$objs $o"
done
gcc $FLAGS -I"$ROOT/oracle/fftw_shim" -I"$REF" -I"$ROOT/include" -c "$HERE/fe_dropin.c" -o "$OUT/fe_dropin.o"
gcc -std=gnu99 -O2 -c "$ROOT/oracle/fftw_shim/fftw_shim.c" -o "$OUT/fftw_shim.o"
gcc -std=gnu99 -O2 -c "$ROOT/oracle/fe_fft.c" -o "$OUT/fe_fft.o"
CUDA=${CUDA_HOME:-/usr/local/cuda}
gcc -o "$OUT/spidey_gpu" $objs "$OUT/fe_dropin.o" "$OUT/fftw_shim.o" "$OUT/fe_fft.o" \
    -L"$PKG" -lfe -L"$CUDA/lib64" -lcudart -lcufft -Wl,-rpath,"$PKG" -Wl,-rpath,"$CUDA/lib64" -lm
echo "linked $OUT/spidey_gpu"
