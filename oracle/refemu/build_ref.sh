#!/bin/sh
# Builds the reference's own solver (GraphCut.cu + GraphCutKernels.cu, read
# from the reference checkout, unmodified except that each `K<<<g,b>>>(`
# launch is rewritten on the fly to `emu_launch(g,b, K, `) for the CPU
# thread emulator) together with ref_harness.cpp into oracle/_ref/.
# Test infrastructure only: it produces the golden outputs that pin the
# oracle.  Nothing from the reference is written anywhere but oracle/_ref/.
set -e
REF=${GCFG_REFERENCE_DIR:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/../_ref"
if [ ! -f "$REF/GraphCut.cu" ]; then
  echo "reference checkout not found at $REF" >&2
  exit 3
fi
mkdir -p "$OUT"
FLAGS="-O2 -std=c++17 -U_FORTIFY_SOURCE -D_FORTIFY_SOURCE=0 -fcf-protection=none -w"
sed -E 's/([A-Za-z_][A-Za-z0-9_]*)<<<([^>]*)>>>\(/emu_launch(\2, \1, /' "$REF/GraphCut.cu" |
  g++ $FLAGS -x c++ -I "$HERE" -I "$REF" -include cuda_emu.h -c - -o "$OUT/graphcut_ref.o"
g++ $FLAGS -I "$HERE" -c "$HERE/cuda_emu.cpp" -o "$OUT/cuda_emu.o"
g++ $FLAGS -I "$HERE" -I "$REF" -include cuda_emu.h -c "$HERE/ref_harness.cpp" -o "$OUT/ref_harness.o"
g++ -o "$OUT/ref_harness" "$OUT/graphcut_ref.o" "$OUT/cuda_emu.o" "$OUT/ref_harness.o"
echo "$OUT/ref_harness"
