"""Smoke check of the IMEX step (filled in as the step path lands): nothing yet beyond the
banded solve exercised by ``__graft_entry__.smoke``."""


def run() -> None:
    return None
