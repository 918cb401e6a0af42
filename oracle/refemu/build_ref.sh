#!/bin/sh
# Builds the reference's own solver (GraphCut.cu + GraphCutKernels.cu, read
# from the reference checkout, unmodified except that each `K<<<g,b>>>(`
# launch is rewritten on the fly to `emu_launch(g,b, K, `) for the CPU
# thread emulator) together with ref_harness.cpp into oracle/_ref/, and the
# reference's applications that feed it: solveMRF.cu and Application.cu
# (compiled from stdin in app_include/, whose GraphCut.cu declares the host
# API that graphcut_ref.o defines) and multiplyMRF.cpp (plain C++; once as it
# is, the 3600x3600 mode, and once with its DO_RIHANNA switch turned to 0 on
# the fly, the general tiling mode), the reference's DataTerm.cpp with
# dt_harness.cpp (its kernel-density data term), and the solver built with
# NEIGHBORHOOD 8 with ref_harness8.cpp.
# Test infrastructure only: it produces the golden outputs that pin the
# oracle and the tools.  Nothing from the reference is written anywhere but
# oracle/_ref/.
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
for app in solveMRF Application; do
  (cd "$HERE/app_include" && g++ $FLAGS -x c++ -I "$HERE" -I "$REF" -include cuda_emu.h -c - \
      -o "$OUT/${app}_ref.o" < "$REF/$app.cu")
  g++ -o "$OUT/$app" "$OUT/${app}_ref.o" "$OUT/graphcut_ref.o" "$OUT/cuda_emu.o"
done
# the solver again with NEIGHBORHOOD 8 (its header, switched on the fly, is
# streamed ahead of the source; no modified copy is written anywhere)
N8='s/^#define NEIGHBORHOOD 4/#define NEIGHBORHOOD 8/'
{ sed "$N8" "$REF/GraphCut.h"; sed -E 's/([A-Za-z_][A-Za-z0-9_]*)<<<([^>]*)>>>\(/emu_launch(\2, \1, /' "$REF/GraphCut.cu"; } |
  g++ $FLAGS -x c++ -I "$HERE" -I "$REF" -include cuda_emu.h -c - -o "$OUT/graphcut8_ref.o"
{ sed "$N8" "$REF/GraphCut.h"; cat "$HERE/ref_harness8.cpp"; } |
  g++ $FLAGS -x c++ -I "$HERE" -I "$REF" -include cuda_emu.h -c - -o "$OUT/ref_harness8.o"
g++ -o "$OUT/ref_harness8" "$OUT/graphcut8_ref.o" "$OUT/cuda_emu.o" "$OUT/ref_harness8.o"
# the reference's DataTerm namespace (DataTerm.cpp + DataTermKernels.cu) and its driver
(cd "$HERE/app_include" && sed -E 's/([A-Za-z_][A-Za-z0-9_]*)<<<([^>]*)>>>\(/emu_launch(\2, \1, /' "$REF/DataTerm.cpp" |
  g++ $FLAGS -x c++ -I "$HERE" -I "$REF" -include cuda_emu.h -include cutil.h "-Duchar=unsigned char" -c - \
      -o "$OUT/dataterm_ref.o")
g++ $FLAGS -I "$HERE" -c "$HERE/dt_harness.cpp" -o "$OUT/dt_harness.o"
g++ -o "$OUT/dt_harness" "$OUT/dataterm_ref.o" "$OUT/cuda_emu.o" "$OUT/dt_harness.o"
g++ -O2 -w -o "$OUT/multiplyMRF" "$REF/multiplyMRF.cpp"
sed 's/^#define DO_RIHANNA 1/#define DO_RIHANNA 0/' "$REF/multiplyMRF.cpp" | g++ -O2 -w -x c++ - -o "$OUT/multiplyMRF_tile"
echo "$OUT/ref_harness"
