"""Physical systems: plugin objects with ``DOF``, ``potential`` (a C expression in x1..xDOF),
``userCode`` (C source pasted before the kernel) and operator strings, exactly the contract
of the reference's FeynSimul/physical_systems/__init__.py:1-18."""
