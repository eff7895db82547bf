#!/bin/bash
# Size sweep of the benchmark command line, as the reference runs it (build_me.sh): for
# count = 256, 512, ..., up to max_count it sorts count x count and 2*count x count keys
# (2^16 .. 2^29 at the default 16384), `trials` runs of `iterations` sorts each, every run
# printing the reference's statistics lines for uint, float and double.
#
#   sweep.sh [max_count=16384] [trials=3] [iterations=10]
#
# The command line must be built first (python -c "import __graft_entry__ as g; g.build()").
# Stops at the first run that fails (wrong result, no sm_103 GPU, bad arguments).
set -e
PKG=$(cd "$(dirname "$0")/.." && pwd)
BIN="$PKG/quicksort"
MAX=${1:-16384}
TRIALS=${2:-3}
ITERS=${3:-10}
if [ ! -x "$BIN" ]; then
  echo "$BIN is missing: build it with __graft_entry__.build()"
  exit 1
fi
count=256
while [ "$count" -le "$MAX" ]; do
  for width in "$count" $((count * 2)); do
    for trial in $(seq 1 "$TRIALS"); do
      echo "-------------- Trial $trial ---- $width x $count ----------"
      "$BIN" "$ITERS" gpu nvidia "$width" "$count" show_cl
    done
  done
  count=$((count * 2))
done
