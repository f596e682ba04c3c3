#!/bin/sh
# Builds oracle/_ref/librefemu.so: the reference's own OpenCL kernel source
# (src/kernels{1,2,3}D.cl) compiled as C++ and driven in the reference's host
# order by oracle/ref_driver.cpp.  Test infrastructure only.
#
# The reference is read where it lies: the directory TOPEFFT_REFERENCE names,
# else a checkout named "reference" beside this repository; the rewritten
# sources and the library go to oracle/_ref/,
# which is git-ignored.  When the reference tree is absent but oracle/_ref/
# already holds the rewritten sources (copied along with the working tree),
# only the compile step runs.  Exit status 3 means "reference unavailable".
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${TOPEFFT_REFERENCE:-$HERE/../../reference}
OUT="$HERE/_ref"
mkdir -p "$OUT"
if [ -d "$REF/src" ]; then
    for d in 1 2 3; do
        sed -e 's/#pragma OPENCL.*//' \
            -e 's/__kernel//g;s/__global//g;s/__private//g' \
            -e 's/(double\(2\|4\|8\|16\))(/double\1(/g' \
            -e 's/\bnew\b/new_/g' \
            "$REF/src/kernels${d}D.cl" > "$OUT/k${d}d.cpp"
    done
fi
for d in 1 2 3; do
    [ -f "$OUT/k${d}d.cpp" ] || { echo "reference kernels unavailable" >&2; exit 3; }
done
${CXX:-g++} -O2 -fopenmp -ffp-contract=off -fPIC -shared -w \
    -I"$HERE" -I"$OUT" "$HERE/ref_driver.cpp" -o "$OUT/librefemu.so.tmp"
mv "$OUT/librefemu.so.tmp" "$OUT/librefemu.so"
