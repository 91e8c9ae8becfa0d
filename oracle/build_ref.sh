#!/bin/sh
# Compiles the reference's own CPU-runnable ABEA code into oracle/_ref/libref.so
# (test infrastructure: pins the oracle restatement).  Sources are read where
# they lie in the reference checkout; outputs go only to oracle/_ref/.
#   FPGA/code/device/align_swi.cl            fill kernel, compiled as C
#   FPGA/code/host/src/align_swi.cpp:959-1314 host traceback/QC, compiled as C++
# The checkout's location comes from ABEA_REFERENCE_DIR; without it, or when the
# sources are not there, the step is skipped.  The checkout's path is recorded in
# _ref/source_dir for the tests that read the reference's golden dump.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${ABEA_REFERENCE_DIR:-}
OUT="$HERE/_ref"
if [ -z "$REF" ] || [ ! -f "$REF/FPGA/code/device/align_swi.cl" ]; then
    echo "build_ref: ABEA_REFERENCE_DIR unset or without the reference sources; skipped"
    exit 0
fi
mkdir -p "$OUT"
printf '%s\n' "$REF" > "$OUT/source_dir"
gcc -std=gnu11 -fgnu89-inline -O2 -ffp-contract=off -fPIC -w -include "$HERE/ref_shim_kernel.h" \
    -x c -c "$REF/FPGA/code/device/align_swi.cl" -o "$OUT/align_swi.o"
sed -n '959,1314p' "$REF/FPGA/code/host/src/align_swi.cpp" > "$OUT/host_post.inc"
g++ -O2 -ffp-contract=off -fPIC -w -I"$OUT" -c "$HERE/ref_wrapper.cpp" -o "$OUT/ref_wrapper.o"
g++ -shared -o "$OUT/libref.so" "$OUT/align_swi.o" "$OUT/ref_wrapper.o" -lm
echo "build_ref: built $OUT/libref.so"
