#!/bin/sh
# Builds oracle/_ref/libref_demsph.so: the reference's own solver compiled for
# the CPU, used only to pin the FP64 oracle and to generate tests/golden/.
#
# The reference's kernels are launched with CUDA's <<<grid, block>>> syntax,
# which a host compiler cannot parse, so the sources are streamed (never
# copied to disk) through one sed expression that turns each launch
#     kernel << <grid, block >> > (args)
# into the shim's sequential emulator call
#     refshim::launch(grid, block, kernel)(args)
# and then compiled as one C++ translation unit together with
# oracle/ref_harness.cpp.  Everything else - the CUDA runtime calls, thrust and
# the built-in index variables - comes from oracle/refshim/.
#
# Needs the reference sources at $REF (default: a directory "reference" beside
# the repository).  Runs where they exist; the output is a checker, not part
# of the product.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${REF:-$(cd "$HERE/../.." && pwd)/reference}
OUT="$HERE/_ref"
if [ ! -d "$REF/core" ]; then
    echo "build_ref.sh: reference sources not found at $REF/core" >&2
    exit 2
fi
mkdir -p "$OUT"
{
    for f in "$REF/core/dataBase.cpp" "$REF/core/solverBase.cpp" \
             "$REF/core/neighborSearch.cu" "$REF/core/integrate.cu" "$HERE/ref_harness.cpp"; do
        cat "$f"
        echo    # the reference's files do not all end in a newline
    done
} | sed -E 's/([A-Za-z_][A-Za-z_0-9]*) << <([A-Za-z_][A-Za-z_0-9]*), ([A-Za-z_][A-Za-z_0-9]*) >> > \(/refshim::launch(\2, \3, \1)(/g' \
  | g++ -std=c++17 -O2 -fPIC -shared -ffp-contract=off -w \
        -I"$HERE/refshim" -I"$REF/core" -include "$HERE/refshim/prelude.h" \
        -x c++ - -o "$OUT/libref_demsph.so"
echo "built $OUT/libref_demsph.so"
