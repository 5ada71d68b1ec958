#!/usr/bin/env bash
# Test infrastructure: compiles the reference FAME sources (the oracle) into
# shared libraries under oracle/_ref together with oracle/ref_driver.cpp.
#
# Stage 1 (only where the reference tree is present: FAME_REFERENCE_DIR, by
# default a checkout named "reference" beside this repository): copy the files
# the matching path needs into oracle/_ref/src (git-ignored).
# Stage 2 (also on machines without the reference tree, from the staged
# copy): one build per constant set, each from its own copy of the sources
# with CONST.h patched (CORENUM, READLEN and MAXPDIST are #defines or
# constexprs in CONST.h:35-42 that -D cannot override; quoted includes find
# the copy's own CONST.h):
#   libfame_ref.so        READLEN 100, MAXPDIST 550 (the reference's values)
#   libfame_ref_rl150.so  READLEN 150, MAXPDIST 550
#   libfame_ref_pd400.so  READLEN 100, MAXPDIST 400
# CORENUM is the core count of the machine that builds them.  The reference
# Makefile's -march=native is passed where the compiler accepts it.  Nothing
# is written outside oracle/_ref.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
SRC="$OUT/src"
REF="${FAME_REFERENCE_DIR:-$HERE/../../reference}"
CORES="${FAME_REF_CORENUM:-$(nproc)}"

mkdir -p "$OUT"
if [ -f "$REF/ReadQueue.cpp" ]; then
  rm -rf "$SRC"
  mkdir -p "$SRC/spaced_nthash" "$SRC/gzstream" "$SRC/hopscotch-map/include/tsl"
  for f in main.cpp CONST.h CONST.cpp structs.h RefGenome.h RefGenome.cpp RefReader_istr.h RefReader_istr.cpp \
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
ARCHFLAG=""
if echo 'int main(){return 0;}' | g++ -march=native -x c++ - -o /dev/null 2>/dev/null; then
  ARCHFLAG="-march=native"
fi

build_variant() {   # readlen maxpdist library-name
  local rl="$1" pd="$2" name="$3"
  local vs="$OUT/src_${rl}_${pd}"
  rm -rf "$vs"
  cp -r "$SRC" "$vs"
  sed -i -E "s/^#define CORENUM .*/#define CORENUM ${CORES}/" "$vs/CONST.h"
  sed -i -E "s/^constexpr unsigned int READLEN = .*;/constexpr unsigned int READLEN = ${rl};/" "$vs/CONST.h"
  sed -i -E "s/^constexpr uint32_t MAXPDIST = .*;/constexpr uint32_t MAXPDIST = ${pd};/" "$vs/CONST.h"
  local flags="-std=c++14 -O3 $ARCHFLAG -fopenmp -fPIC -w -Dprivate=public -I$vs -I$vs/hopscotch-map/include/tsl"
  # ref_driver.cpp is compiled from a copy inside the variant's tree so that its
  # quoted includes resolve to the variant's CONST.h
  cp "$HERE/ref_driver.cpp" "$vs/ref_driver.cpp"
  g++ $flags -shared -o "$OUT/$name.tmp" \
      "$vs/ref_driver.cpp" "$vs/RefGenome.cpp" "$vs/RefReader_istr.cpp" "$vs/Read.cpp" \
      "$vs/CONST.cpp" "$vs/DnaBitStr.cpp" "$vs/gzstream/gzstream.C" -lz
  mv "$OUT/$name.tmp" "$OUT/$name"
  echo "build_ref: built $OUT/$name (CORENUM=$CORES READLEN=$rl MAXPDIST=$pd ${ARCHFLAG:-no -march=native})"
}

pids=()
build_variant 100 550 libfame_ref.so & pids+=($!)
build_variant 150 550 libfame_ref_rl150.so & pids+=($!)
build_variant 100 400 libfame_ref_pd400.so & pids+=($!)
rc=0
for p in "${pids[@]}"; do wait "$p" || rc=1; done
exit $rc
