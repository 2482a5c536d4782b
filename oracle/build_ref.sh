#!/bin/sh
# Builds oracle/_ref/libsoft_ref.so from the reference's own SOFT 1.0 C sources
# (read in place under the reference tree, never copied) plus the project's
# fftw3.h shim and harness, and oracle/_ref/libblitz_ref.so from the reference's
# cylindrical-domain headers and representation-distance loop on its vendored
# Blitz. Test infrastructure only; needs the reference tree.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${ETTK_REFERENCE_ROOT:-/root/reference}"
SOFT="$REF/external/soft-1.0"
OUT="$HERE/_ref"
if [ ! -d "$SOFT" ]; then
  echo "build_ref: $SOFT not found; skipping the SOFT reference build" >&2
  exit 0
fi
mkdir -p "$OUT/obj"
SRCS="cospmls csecond fft_grids FFTcode FST_semi_memo indextables makeWigner naive_synthesis newFCT oddweights OURmods OURperms permroots primitive primitive_FST rotate_so3 seminaive utils_so3 weights soft_fftw so3_correlate_fftw wignerTransforms_fftw utils_vec_cx"
for s in $SRCS; do
  gcc -O2 -fPIC -w -I"$HERE/shim" -I"$SOFT" -c "$SOFT/$s.c" -o "$OUT/obj/$s.o" &
done
gcc -O2 -fPIC -w -I"$HERE/shim" -I"$SOFT" -c "$HERE/shim/soft_ref_wrap.c" -o "$OUT/obj/soft_ref_wrap.o" &
g++ -O2 -fPIC -std=c++17 -I"$HERE/shim" -c "$HERE/shim/fftw_shim.cpp" -o "$OUT/obj/fftw_shim.o" &
g++ -O2 -fPIC -std=c++17 -c "$HERE/fft64.cpp" -o "$OUT/obj/fft64.o" &
wait
g++ -shared -o "$OUT/libsoft_ref.so" "$OUT"/obj/*.o -lm
echo "built $OUT/libsoft_ref.so"
# The reference's cylindrical-domain classes (header-only), the representation-distance loop, the class-selection
# rules and the Fourier filter / spectrum normalisation / CCF distance expressions, on its vendored Blitz 0.9,
# behind C harnesses.
BLITZ="$REF/external/blitz-0.9"
if [ -d "$BLITZ/blitz" ]; then
  g++ -O2 -fPIC -std=c++11 -w -ffp-contract=off -shared -I"$BLITZ" -I"$REF/inc" \
    "$HERE/shim/cyl_ref_wrap.cpp" "$HERE/shim/repr_blitz_wrap.cpp" "$HERE/shim/clustering_blitz_wrap.cpp" \
    "$HERE/shim/filter_blitz_wrap.cpp" \
    -o "$OUT/libblitz_ref.so"
  echo "built $OUT/libblitz_ref.so"
fi
