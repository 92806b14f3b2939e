#!/bin/bash
# Install the reference package (pure Python) into baseline/_ref, where
# bench.py's reference arm imports it to time the reference's own code path.
# Usage (from the repository root):
#   bash oracle/install_reference.sh [reference-checkout]
# (default: the build container's checkout at /root/reference; without a
# checkout it does nothing).  The checkout may be read-only: it is copied to
# a scratch folder first, because setuptools writes build metadata next to
# setup.py.  No network: the install takes no dependencies (numpy and scipy
# are already present).
set -euo pipefail
src="${1:-/root/reference}"
if [ ! -f "$src/setup.py" ]; then
  echo "no reference checkout at $src; nothing installed"
  exit 0
fi
here="$(cd "$(dirname "$0")/.." && pwd)"
tmp="$(mktemp -d)"
trap 'rm -rf "$tmp"' EXIT
cp -r "$src" "$tmp/qspectra_src"
python -m pip install --quiet --no-index --no-build-isolation --no-deps \
    --target "$here/baseline/_ref" "$tmp/qspectra_src"
echo "installed into $here/baseline/_ref"
