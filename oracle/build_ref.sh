#!/bin/bash
# Builds the reference program (cuda-version/ of JuZhenCS/gene-sequences-de-redundancy)
# from its own three source files, unmodified, into oracle/_ref/.  Test
# infrastructure only: it produces the golden outputs of tests/golden/.
#
#   oracle/build_ref.sh stage   copy main.cu, func.cu, func.h from the reference
#                               tree (read-only; its root in $GSDR_REFERENCE)
#                               into oracle/_ref/src/
#   oracle/build_ref.sh build   nvcc them for sm_103a into oracle/_ref/cluster_ref_<L>
#                               for each MAX_LENGTH L given in $GSDR_REF_MAXLEN
#
# oracle/_ref/ is git-ignored: neither the copied sources nor the binaries are
# part of this repository.  Staging happens where the reference tree is
# mounted; building and running need a GPU machine with nvcc.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
out="$here/_ref"
src="$out/src"
ref="${GSDR_REFERENCE:-}"
case "${1:-build}" in
  stage)
    [ -n "$ref" ] || { echo "set GSDR_REFERENCE to the reference tree's root" >&2; exit 2; }
    mkdir -p "$src"
    for f in main.cu func.cu func.h; do
      cp "$ref/cuda-version/$f" "$src/$f"
    done
    echo "staged reference sources into $src"
    ;;
  build)
    [ -f "$src/func.cu" ] || { echo "no staged sources in $src (run: $0 stage)" >&2; exit 2; }
    for L in ${GSDR_REF_MAXLEN:-2048 12288}; do
      nvcc -O3 -gencode arch=compute_103a,code=sm_103a -w \
        "$src/main.cu" "$src/func.cu" -DMAX_LENGTH="$L" -o "$out/cluster_ref_$L"
      echo "built $out/cluster_ref_$L"
    done
    ;;
  *)
    echo "usage: $0 stage|build" >&2; exit 2 ;;
esac
