#!/usr/bin/env bash
# Test infrastructure: compiles the reference FAME sources (the oracle) into
# oracle/_ref/libfame_ref.so together with oracle/ref_driver.cpp.
#
# Stage 1 (only where the reference tree is present, FAME_REFERENCE_DIR,
# default /root/reference): copy the files the matching path needs into
# oracle/_ref/src (git-ignored) and set CORENUM (a #define in CONST.h:38 that
# -D cannot override) to the core count of the machine that runs it.
# Stage 2 (also on machines without the reference tree, from the staged
# copy): compile.  Nothing is written outside oracle/_ref.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
SRC="$OUT/src"
REF="${FAME_REFERENCE_DIR:-/root/reference}"
CORES="${FAME_REF_CORENUM:-$(nproc)}"
READLEN="${FAME_REF_READLEN:-100}"
MAXPDIST="${FAME_REF_MAXPDIST:-550}"

mkdir -p "$OUT"
if [ -f "$REF/ReadQueue.cpp" ]; then
  rm -rf "$SRC"
  mkdir -p "$SRC/spaced_nthash" "$SRC/gzstream" "$SRC/hopscotch-map/include/tsl"
  for f in CONST.h CONST.cpp structs.h RefGenome.h RefGenome.cpp RefReader_istr.h RefReader_istr.cpp \
           ReadQueue.h ReadQueue.cpp Read.h Read.cpp ShiftAnd.h LevenshtDP.h BandedMatrix.h \
           DnaBitStr.h DnaBitStr.cpp BitFunctions.h; do
    cp "$REF/$f" "$SRC/$f"
  done
  cp "$REF/spaced_nthash/nthash.hpp" "$SRC/spaced_nthash/"
  cp "$REF/gzstream/gzstream.h" "$REF/gzstream/gzstream.C" "$SRC/gzstream/"
  cp "$REF"/hopscotch-map/include/tsl/*.h "$SRC/hopscotch-map/include/tsl/"
  chmod -R u+w "$SRC"
fi
if [ ! -f "$SRC/ReadQueue.cpp" ]; then
  echo "build_ref: reference sources not available (neither $REF nor a staged copy)" >&2
  exit 3
fi
# per-machine thread count, read length and pair distance (CONST.h:35, 38, 42)
sed -i -E "s/^#define CORENUM .*/#define CORENUM ${CORES}/" "$SRC/CONST.h"
sed -i -E "s/^constexpr unsigned int READLEN = .*;/constexpr unsigned int READLEN = ${READLEN};/" "$SRC/CONST.h"
sed -i -E "s/^constexpr uint32_t MAXPDIST = .*;/constexpr uint32_t MAXPDIST = ${MAXPDIST};/" "$SRC/CONST.h"

CXXFLAGS="-std=c++14 -O3 -fopenmp -fPIC -w -Dprivate=public -I$SRC -I$SRC/hopscotch-map/include/tsl"
g++ $CXXFLAGS -shared -o "$OUT/libfame_ref.so" \
    "$HERE/ref_driver.cpp" "$SRC/RefGenome.cpp" "$SRC/RefReader_istr.cpp" "$SRC/Read.cpp" \
    "$SRC/CONST.cpp" "$SRC/DnaBitStr.cpp" "$SRC/gzstream/gzstream.C" -lz
echo "build_ref: built $OUT/libfame_ref.so (CORENUM=$CORES READLEN=$READLEN MAXPDIST=$MAXPDIST)"
