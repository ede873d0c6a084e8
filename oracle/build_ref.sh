#!/usr/bin/env bash
# Builds the reference's own C++ EPG kernel (src/torchsim/_epg_cpu.cpp) from its
# sources, out of tree, into oracle/_ref/. It is test infrastructure: the
# checker and the timed CPU baseline, never part of the product.
#
# The flags are the reference's own (CMakeLists.txt:48-53): -O3 with
# floating-point contraction off, so the build reproduces its FP32 results bit
# for bit. It needs only the CPython headers; the reference's cmake project is
# not used.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
# The reference checkout is the argument, else $TORCHSIM_REFERENCE, else the
# container's read-only checkout at /root/reference. Where none of them holds
# the sources (a host without the checkout), nothing is built and the CPU
# baseline runs the oracle's port.
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
ref="${1:-${TORCHSIM_REFERENCE:-/root/reference}}"
src="$ref/src/torchsim/_epg_cpu.cpp"
if [[ ! -f "$src" ]]; then
    echo "reference sources not found at $ref; nothing built" >&2
    exit 0
fi
out="$here/_ref"
mkdir -p "$out"
inc="$(python3 -c 'import sysconfig; print(sysconfig.get_paths()["include"])')"
suffix="$(python3 -c 'import sysconfig; print(sysconfig.get_config_var("EXT_SUFFIX"))')"
target="$out/_epg_cpu$suffix"
if [[ -f "$target" && "$target" -nt "$src" ]]; then
    exit 0
fi
g++ -std=c++17 -O3 -ffp-contract=off -shared -fPIC -pthread \
    -I"$inc" -I"$ref/src/torchsim" "$src" -o "$target.tmp"
mv "$target.tmp" "$target"
echo "built $target"
