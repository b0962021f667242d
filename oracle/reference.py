"""Where the reference's source tree is, for the recipes that compile it
(``make -C oracle ref``, ``make -C tests/host binding-check``) — TEST
INFRASTRUCTURE.

``LIGHTFEM_REFERENCE`` names the checkout.  Without it, the read-only mount that
this repository's golden fixtures were generated from is used when it exists.
``None`` means no reference tree on this machine: the recipes that need one are
skipped, and everything else reads the committed fixtures under tests/golden/.
"""

from __future__ import annotations

import os

_MOUNT = "/root/reference"


def reference_root() -> str | None:
    root = os.environ.get("LIGHTFEM_REFERENCE") or _MOUNT
    return root if os.path.isdir(os.path.join(root, "src")) else None


def make_args() -> list[str]:
    """``REF=<root>`` for the Makefiles, or an empty list without a reference."""
    root = reference_root()
    return [f"REF={root}"] if root else []
