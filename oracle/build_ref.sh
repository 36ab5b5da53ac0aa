#!/bin/sh
# Builds the reference CPU implementation of the full-pairwise stage from the
# ClustalW 2.0.11 sources where they lie (read-only) and links it with
# oracle/ref_harness.cpp. TEST INFRASTRUCTURE ONLY: outputs go to oracle/_ref/
# (git-ignored). Needs the reference tree; exits 0 with a note when it is absent.
#
# The reference's autoconf step is not run. It would only contribute two
# configure-time definitions, which this recipe supplies itself: OS_UNIX=1
# (config.h on Linux) and the CLUSTALW_NAME/CLUSTALW_VERSION macros of
# src/clustalw_version.h.in.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
SRC=${CLUSTALW_REF_SRC:-/root/reference/CPU/clustalw-2.0.11/src}
OUT="$HERE/_ref"
if [ ! -f "$SRC/pairwise/FullPairwiseAlign.cpp" ]; then
    echo "build_ref: reference sources not present; skipping"
    exit 0
fi
mkdir -p "$OUT/obj" "$OUT/include"
printf '#define CLUSTALW_NAME "ClustalW"\n#define CLUSTALW_VERSION "2.0.11"\n' > "$OUT/include/clustalw_version.h"
CXX=${CXX:-g++}
FLAGS="-O2 -std=gnu++98 -w -DOS_UNIX=1 -I$SRC -I$OUT/include"
UNITS="pairwise/FullPairwiseAlign pairwise/FastPairwiseAlign substitutionMatrix/SubMatrix general/UserParameters
general/Utility alignment/Alignment alignment/Sequence general/SymMatrix
general/VectorOutOfRange general/InvalidCombination general/DebugLog general/Stats
general/ClustalWResources general/OutputFile fileInput/FileReader fileInput/FileParser
fileInput/PearsonFileParser fileInput/InFileStream fileInput/MSFFileParser
fileInput/PIRFileParser fileInput/RSFFileParser fileInput/GDEFileParser
fileInput/ClustalFileParser fileInput/EMBLFileParser tree/NJTree
tree/UnRootedClusterTree tree/ClusterTree tree/ClusterTreeOutput tree/RandomGenerator"
OBJS=""
for u in $UNITS; do
    o="$OUT/obj/$(basename "$u").o"
    OBJS="$OBJS $o"
    if [ ! -f "$o" ] || [ "$SRC/$u.cpp" -nt "$o" ]; then
        $CXX $FLAGS -c "$SRC/$u.cpp" -o "$o" &
    fi
done
wait
$CXX -O2 -std=gnu++11 -w -DOS_UNIX=1 -I"$SRC" -I"$OUT/include" "$HERE/ref_harness.cpp" $OBJS -o "$OUT/refharness"
echo "build_ref: built $OUT/refharness"
