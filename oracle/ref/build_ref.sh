#!/bin/sh
# Test infrastructure only.  Compiles the reference's vendored URDF parser (urdfdom + tinyxml,
# third/urdf_parser under the reference checkout) with oracle/ref/urdf_dump.cpp into
# oracle/_ref/urdf_dump.  Reads the sources where they lie; writes only into oracle/_ref/.
# Usage: oracle/ref/build_ref.sh [reference_root]
#   reference_root: the argument, else $PLAINMP_REF, else the checkout's location in the build
#   container (/root/reference).  Exits 1 without building when the parser sources are absent.
set -e
REF=${1:-${PLAINMP_REF:-/root/reference}}
U="$REF/third/urdf_parser"
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/../_ref"
[ -d "$U/src" ] || { echo "reference urdf parser not found at $U" >&2; exit 1; }
mkdir -p "$OUT"
g++ -std=c++14 -O2 -I"$U/include" -I"$U/tinyxml" \
  "$U/src/pose.cpp" "$U/src/model.cpp" "$U/src/link.cpp" "$U/src/joint.cpp" \
  "$U/tinyxml/tinystr.cpp" "$U/tinyxml/tinyxml.cpp" "$U/tinyxml/tinyxmlerror.cpp" "$U/tinyxml/tinyxmlparser.cpp" \
  "$HERE/urdf_dump.cpp" -o "$OUT/urdf_dump"
echo "built $OUT/urdf_dump"
