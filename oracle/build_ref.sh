#!/bin/sh
# Compile the reference's reconstruction sources in place against the
# stand-in headers in oracle/ref_shim, into oracle/_ref/libmuto_ref.so (its
# MutoFile into oracle/_ref/libmuto_ref_file.so, its command-line program
# into oracle/_ref/muto_ref_cli).
# Only possible where the reference tree is mounted; test infrastructure only.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
# the reference's source tree: $MUTO_REFERENCE, else "reference" beside this repository
REF=${MUTO_REFERENCE:-$(cd "$HERE/../.." && pwd)/reference}
[ -d "$REF/src" ] || { echo "reference sources not found at $REF" >&2; exit 2; }
mkdir -p "$HERE/_ref"
g++ -O2 -std=c++14 -fPIC -shared -fopenmp -ffp-contract=off -fno-fast-math -w \
    -I "$HERE/ref_shim" -I "$REF/include" \
    "$REF/src/MutoSiddon.cpp" "$REF/src/MutoPoCA.cpp" "$REF/src/MutoMLSD.cpp" "$REF/src/MutoMAP.cpp" \
    "$REF/src/MutoPoCut.cpp" "$REF/src/MutoSLR.cpp" "$REF/src/MutoSLRIter.cpp" \
    "$HERE/ref_harness.cpp" -o "$HERE/_ref/libmuto_ref.so"
# the reference's MutoFile (raw-hit reader and image files) on its own: the
# reconstruction harness above provides its own loadImage
g++ -O2 -std=c++14 -fPIC -shared -ffp-contract=off -fno-fast-math -w \
    -I "$HERE/ref_shim" -I "$REF/include" \
    "$REF/src/MutoFile.cpp" "$HERE/ref_file_harness.cpp" -o "$HERE/_ref/libmuto_ref_file.so"
# the reference's command-line program (MuToTest.cpp) over all of the above
g++ -O2 -std=c++14 -fopenmp -ffp-contract=off -fno-fast-math -w \
    -I "$HERE/ref_shim" -I "$REF/include" \
    "$REF/MuToTest.cpp" "$REF/src/MutoFile.cpp" "$REF/src/MutoSiddon.cpp" "$REF/src/MutoPoCA.cpp" \
    "$REF/src/MutoMLSD.cpp" "$REF/src/MutoMAP.cpp" "$REF/src/MutoPoCut.cpp" "$REF/src/MutoSLR.cpp" \
    "$REF/src/MutoSLRIter.cpp" -o "$HERE/_ref/muto_ref_cli"
echo "built $HERE/_ref/libmuto_ref.so $HERE/_ref/libmuto_ref_file.so $HERE/_ref/muto_ref_cli"
