#!/usr/bin/env bash
# Build the relxill reference's own C/C++ sources into oracle/_ref/ as a
# shared library, for use as a checker only (it validates the C restatement
# in oracle/relx_oracle.c and generates tests/golden/ fixtures).
#
# The reference does not build as shipped: it needs cfitsio, FFTW3 and a
# generated XSPEC wrapper.  This recipe compiles its unmodified sources where
# they lie, against the stand-ins in oracle/shim/ (fitsio.h, fftw3.h,
# xsTypes.h, config.h; implementations oracle/fitsio_lite.c and
# oracle/fft_lite.c), and runs the reference's own wrapper generator
# (src/create_wrapper_xspec.py) into oracle/_ref/gen/.  Nothing is written
# outside oracle/_ref/.  Needs the reference sources (REF_SRC); skipped
# quietly when they are absent.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
# the reference's sources beside the repository unless REF_SRC names them
REF_SRC="${REF_SRC:-$HERE/../../reference/src}"
OUT="$HERE/_ref"
if [ ! -f "$REF_SRC/Relxill.cpp" ]; then
  echo "build_ref: reference sources not found at $REF_SRC; skipping" >&2
  exit 0
fi
mkdir -p "$OUT/gen" "$OUT/obj"
cat "$REF_SRC/modelfiles/lmodel_relxill_public.dat" "$REF_SRC/modelfiles/lmodel_relxill_devel.dat" > "$OUT/gen/lmodel_relxill.dat"
python3 "$REF_SRC/create_wrapper_xspec.py" "$OUT/gen/lmodel_relxill.dat" "$OUT/gen/xspec_wrapper_lmodels.cpp" > "$OUT/gen/wrapper.log"
INC="-I$HERE/shim -I$OUT/gen -I$REF_SRC"
CFLAGS="-O2 -fPIC -std=c99 -D_GNU_SOURCE -w $INC"
CXXFLAGS="-O2 -fPIC -std=c++17 -w $INC"
objs=()
pids=()
for f in "$REF_SRC"/*.c; do
  b=$(basename "$f" .c)
  gcc $CFLAGS -c "$f" -o "$OUT/obj/$b.o" & pids+=($!)
  objs+=("$OUT/obj/$b.o")
done
for f in "$REF_SRC"/*.cpp; do
  b=$(basename "$f" .cpp)
  [ "$b" = "test_sta" ] && continue
  g++ $CXXFLAGS -c "$f" -o "$OUT/obj/$b.o" & pids+=($!)
  objs+=("$OUT/obj/$b.o")
done
g++ $CXXFLAGS -c "$OUT/gen/xspec_wrapper_lmodels.cpp" -o "$OUT/obj/xspec_wrapper_lmodels.o" & pids+=($!)
g++ $CXXFLAGS -c "$HERE/ref_driver.cpp" -o "$OUT/obj/ref_driver.o" & pids+=($!)
gcc -O2 -fPIC -std=c99 -I"$HERE" -c "$HERE/fitsio_lite.c" -o "$OUT/obj/fitsio_lite.o" & pids+=($!)
gcc -O2 -fPIC -std=c99 -I"$HERE" -c "$HERE/fft_lite.c" -o "$OUT/obj/fft_lite.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
g++ -shared -o "$OUT/librelxill_ref.so" "${objs[@]}" "$OUT/obj/xspec_wrapper_lmodels.o" \
    "$OUT/obj/ref_driver.o" "$OUT/obj/fitsio_lite.o" "$OUT/obj/fft_lite.o" -lm
echo "build_ref: wrote $OUT/librelxill_ref.so (flags: $CXXFLAGS)"
