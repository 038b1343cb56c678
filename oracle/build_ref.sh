#!/bin/sh
# Builds oracle/_ref/corsika_dump: oracle/corsika_dump.c over the reference's
# own eventio reader, compiled from its sources where they lie under the
# reference tree (test infrastructure; nothing is copied into this repo).
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
# The reference root is the argument, else $ROBAST_REFERENCE, else a
# checkout named "reference" beside this repository.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-${ROBAST_REFERENCE:-$HERE/../../reference}}
if [ ! -d "$REF/src/bernlohr" ]; then
  echo "reference tree not present: oracle/_ref not built"
  exit 0
fi
OUT="$HERE/_ref"
mkdir -p "$OUT"
gcc -O1 -w -I "$REF/include/bernlohr" -o "$OUT/corsika_dump" "$HERE/corsika_dump.c" \
    "$REF/src/bernlohr/eventio.c" "$REF/src/bernlohr/io_simtel.c" "$REF/src/bernlohr/fileopen.c" \
    "$REF/src/bernlohr/straux.c" "$REF/src/bernlohr/warning.c" -lm
echo "$OUT/corsika_dump"
