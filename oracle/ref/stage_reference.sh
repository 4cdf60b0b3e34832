#!/bin/sh
# Stages aphros's sources as the installed reference under baseline/_ref/
# (git-ignored; it travels with the working tree so the reference's own CPU
# code can be compiled by oracle/ref/Makefile wherever the tests or the
# benchmark's reference arm run).  aphros has no Python package to
# pip-install, so the install is this copy of its C++ source tree.
#
#   sh oracle/ref/stage_reference.sh [path/to/aphros]   (default /root/reference)
set -e
SRC=${1:-/root/reference}
HERE=$(cd "$(dirname "$0")/../.." && pwd)
DST="$HERE/baseline/_ref/aphros"
test -d "$SRC/src/linear" || { echo "no aphros sources at $SRC" >&2; exit 1; }
mkdir -p "$DST"
rm -rf "$DST/src"
cp -r "$SRC/src" "$DST/src"
chmod -R u+w "$DST"
echo "staged $SRC/src -> $DST/src"
