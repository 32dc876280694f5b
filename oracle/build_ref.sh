#!/bin/sh
# Build recipe for the reference binaries used to pin the oracle (TEST INFRASTRUCTURE ONLY).
# Compiles the reference's own sources where they lie (read-only) and writes only into
# oracle/_ref/.  No source file is copied or edited.  The two force-includes work around a
# two-phase-lookup error in AMS-DEMO/Individual.h:358-381; -DNO_MPI selects the sequential
# build; -DNDEBUG removes an assert with a side effect (simlib/simulator.cpp:563);
# -ffp-contract=off keeps a*b+c unfused on every host (gcc fuses by default on aarch64).
#   ekgSim_ref : the unmodified ekgSim CLI (main.cpp, sim.cpp, simlib, copyOfLibs)
#   ref_dump   : oracle/ref_dump.cpp linked with simlib, writes raw FP64 results
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
# the reference sources: the first argument, else $EKGSIM_REFERENCE, else a checkout named
# "reference" beside this repository
REF=${1:-${EKGSIM_REFERENCE:-$(dirname "$(dirname "$HERE")")/reference}}
OUT="$HERE/_ref"
mkdir -p "$OUT"
FLAGS="-O2 -std=c++11 -DNDEBUG -DNO_MPI -ffp-contract=off -w -I$REF -I$REF/copyOfLibs -I$REF/simlib"
g++ $FLAGS -include vector -include iostream -include "$REF/AMS-DEMO/VectorArithmetics.h" \
    -o "$OUT/ekgSim_ref.tmp" "$REF/main.cpp" "$REF/sim.cpp" "$REF/simlib/simulator.cpp" \
    "$REF/simlib/lib_main.cpp" "$REF/copyOfLibs/Ini.cpp" "$REF/copyOfLibs/Arguments.cpp" \
    "$REF/copyOfLibs/Random.cpp" -ldl &
g++ $FLAGS -o "$OUT/ref_dump.tmp" "$HERE/ref_dump.cpp" "$REF/simlib/simulator.cpp" \
    "$REF/copyOfLibs/Ini.cpp" &
wait
mv "$OUT/ekgSim_ref.tmp" "$OUT/ekgSim_ref"
mv "$OUT/ref_dump.tmp" "$OUT/ref_dump"
