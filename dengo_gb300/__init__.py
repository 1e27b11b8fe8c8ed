"""GB300 (sm_103a) solvers for Dengo's chemistry/cooling networks.

Network definition (the reference's API): ``chemical_network``,
``reaction_classes``, ``primordial_rates``, ``primordial_cooling``,
``ion_by_ion``, ``networks`` (the shipped networks), ``exceptions``,
``mixin``.  Code generation and build: ``codegen``, ``templates``, ``build``
(one CUDA library per network under ``generated/<name>``; sources in
``csrc``).  Calling the solvers: ``runtime`` (ctypes over the C ABI of
``include/dengo_gb300.h``), ``batching`` (autotuner, CUDA-graph hydro
steps), ``serving`` (continuous-batching request loop), ``sharding``
(cells across ranks).  ``tablefile`` reads and writes the ``.dgt`` table
bundles; ``workloads`` draws seeded synthetic cells.
"""
