#!/usr/bin/env bash
# Builds the reference CPU engine of vakuras/moleculardynamics IN PLACE from
# its own sources (read-only tree given as the required argument $1) into
# oracle/_ref/; the tree's location is recorded in oracle/_ref/source_root for
# the tests that compile reference files themselves.  Test infrastructure only: nothing here is shipped or timed as
# the product.
#
# The reference is Visual Studio 2008 code.  It compiles with g++ unmodified
# given four shims, all generated into oracle/_ref/shim (git-ignored):
#   1. <windows.h>: DWORD and GetTickCount (Global.h:15, cpu/cpumd/Host.cpp:40,130)
#   2. namespace std::tr1 for `using namespace tr1` (common/ConfigParser.h:19)
#   3. forwarding headers whose file NAMES contain the backslash paths used by
#      the reference (`#include "..\..\common\Global.h"`, cpu/common/Device.h:12)
#   4. lower-case forwarding headers for mis-cased includes
#      (common/Getters.h:12-13,26, common/DebugCalculations.h:12,16, ...)
# The reference is built twice:
#   libmdref_neon.so   as shipped: species N, O, NG = neon (common/Constants.h)
#   libmdref_argon.so  the same code with oracle/argon_constants.h
#                      pre-included, which defines CONSTANTS_H first so that
#                      the reference table is replaced by one whose NG slot is
#                      argon (sigma 3.405 A, eps/kB 119.8 K, m 39.948)
# plus the unmodified cpumd program (oracle/_ref/cpumd_neon) for end-to-end
# runs of hostMain.  Precision: real = double (-DEQUI), which is how cpumd is
# configured in cpu/cpumd/cpumd.vcproj:46.
set -euo pipefail
if [ $# -lt 1 ]; then
  echo "usage: build_ref.sh <reference source tree>" >&2
  exit 2
fi
REF=$1
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
SHIM="$OUT/shim"
if [ ! -f "$REF/common/NeighborList.cpp" ]; then
  echo "reference sources not found at $REF" >&2
  exit 2
fi
mkdir -p "$SHIM"
printf '%s\n' "$REF" > "$OUT/source_root"

cat > "$SHIM/windows.h" <<'EOF'
#pragma once
#include <time.h>
typedef unsigned long DWORD;
static inline DWORD GetTickCount(void) {
  struct timespec ts; clock_gettime(CLOCK_MONOTONIC, &ts);
  return (DWORD)(ts.tv_sec * 1000UL + ts.tv_nsec / 1000000UL);
}
EOF
cat > "$SHIM/prelude.h" <<'EOF'
#pragma once
#include <cstring>
#include <cstdlib>
namespace std { namespace tr1 {} }
EOF

fwd() {  # fwd <shim file name> <real path>
  printf '#include "%s"\n' "$2" > "$SHIM/$1"
}
# lower-case names used by the reference
fwd global.h        "$REF/common/Global.h"
fwd constants.h     "$REF/common/Constants.h"
fwd getters.h       "$REF/common/Getters.h"
fwd getters.cpp     "$REF/common/Getters.cpp"
fwd results.h       "$REF/common/Results.h"
fwd loader.h        "$REF/common/Loader.h"
# backslash paths (one file name each) used by cpu/common and cpu/cpumd
for h in Global.h Constants.h arvdwfc.h getters.h ConfigParser.h NeighborList.h \
         Loader.h DebugCalculations.h results.h global.h loader.h; do
  real="$REF/common/$h"
  [ -f "$real" ] || real="$SHIM/$h"
  fwd "..\\..\\common\\$h" "$real"
done
fwd '..\common\Device.h' "$REF/cpu/common/Device.h"
fwd host.h "$REF/cpu/cpumd/Host.h"

CXX=${CXX:-g++}
# -ffp-contract=off: no fused multiply-add, so that x86-64 and aarch64 hosts
# evaluate every expression with the same roundings as the shipped x86 build.
FLAGS="-O2 -std=gnu++14 -fPIC -w -DEQUI -ffp-contract=off -fno-fast-math -I$SHIM -include $SHIM/prelude.h"
SRCS="$REF/common/NeighborList.cpp $REF/common/DebugCalculations.cpp \
      $REF/common/ConfigParser.cpp $REF/common/Loader.cpp $REF/common/Results.cpp \
      $REF/cpu/common/Device.cpp $REF/cpu/cpumd/Host.cpp"

build_variant() {  # build_variant <name> <extra flags>
  local name=$1; shift
  local obj="$OUT/obj_$name"; mkdir -p "$obj"
  local objs=""
  for s in $SRCS "$HERE/ref_harness.cpp"; do
    local o="$obj/$(basename "${s%.*}").o"
    $CXX $FLAGS "$@" -c "$s" -o "$o" &
    objs="$objs $o"
  done
  wait
  $CXX -shared -o "$OUT/libmdref_$name.so" $objs
  $CXX $FLAGS "$@" -c "$REF/cpu/cpumd/Main.cpp" -o "$obj/Main.o"
  local progobjs=""
  for o in $objs; do case "$o" in *ref_harness.o) ;; *) progobjs="$progobjs $o";; esac; done
  $CXX -o "$OUT/cpumd_$name" $progobjs "$obj/Main.o"
}
# equi (cpu/equi/Host.cpp, Statistics.cpp) for chooseVelocities and inverf.
# Two more shims, force-included into those two files only:
#   - RAND_MAX is the value of the platform the reference was written for
#     (Visual C++: 0x7fff).  With glibc's 2^31 - 1, MD_RANDMAX = RAND_MAX + 2
#     (cpu/equi/Host.h:26) overflows int and every draw comes out negative.
#   - rand() replays a stream of draws the test supplies
#     (ref_equi_harness.cpp), instead of the clock-seeded stream of :83.
# <cfloat> is included for DBL_MAX (Statistics.cpp:121), which the Visual C++
# headers provided indirectly.  -fno-builtin keeps the compiler from treating
# the reference's own erf/erfc (Statistics.cpp:175-227) as the library's, and
# -Bsymbolic binds the library's calls to them rather than to libm's.
{
  echo '#pragma once'
  echo '#include <cstdlib>'
  echo '#include <cfloat>'
  echo '#undef RAND_MAX'
  echo '#define RAND_MAX 0x7fff'
  echo 'extern "C" int mdref_replay_rand(void);'
  echo '#define rand() mdref_replay_rand()'
} > "$SHIM/equi_shim.h"
build_equi() {  # build_equi <name> <extra flags>
  local name=$1; shift
  local obj="$OUT/obj_$name"
  local objs=""
  for s in "$REF/cpu/equi/Host.cpp" "$REF/cpu/equi/Statistics.cpp"; do
    local o="$obj/equi_$(basename "${s%.*}").o"
    $CXX $FLAGS -fno-builtin -include "$SHIM/equi_shim.h" "$@" -c "$s" -o "$o" &
    objs="$objs $o"
  done
  $CXX $FLAGS "$@" -c "$HERE/ref_equi_harness.cpp" -o "$obj/ref_equi_harness.o" &
  wait
  local common=""
  for s in $SRCS; do
    case "$s" in *cpumd/Host.cpp) ;; *) common="$common $obj/$(basename "${s%.*}").o";; esac
  done
  $CXX -shared -Wl,-Bsymbolic -o "$OUT/libmdref_equi_$name.so" $objs \
      "$obj/ref_equi_harness.o" $common
}

build_variant neon
build_variant argon -include "$HERE/argon_constants.h"
build_equi neon
build_equi argon -include "$HERE/argon_constants.h"
echo "built $OUT/libmdref_neon.so $OUT/libmdref_argon.so $OUT/cpumd_neon $OUT/cpumd_argon" \
     "$OUT/libmdref_equi_neon.so $OUT/libmdref_equi_argon.so"
