#!/bin/sh
# ORACLE recipe — compiles the reference's own host plan (header-only C++17,
# native-smoke/rns-plan.hpp) together with oracle/ref_plan_dump.cpp into
# oracle/_ref/ref_plan_dump.  Runs only where the reference checkout exists;
# its output feeds tests/golden/make_golden.py.  Nothing of the reference is
# copied into the repository.
set -eu
REF=${REFERENCE_ROOT:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
if [ ! -f "$REF/native-smoke/rns-plan.hpp" ]; then
    echo "reference checkout not found at $REF; skipping oracle/_ref" >&2
    exit 0
fi
mkdir -p "$HERE/_ref"
g++ -std=c++17 -O2 -I "$REF/native-smoke" -o "$HERE/_ref/ref_plan_dump" "$HERE/ref_plan_dump.cpp"
echo "$HERE/_ref/ref_plan_dump"
