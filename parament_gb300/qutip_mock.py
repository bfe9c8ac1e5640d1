"""Stand-in for qutip when it is not installed: only the ``Qobj`` type is
needed, for ``isinstance`` checks (src/python/pyparament/parament/qutip_mock.py:15-16)."""


class Qobj:
    pass
