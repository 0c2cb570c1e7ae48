"""MADAM's node bound (Evaluate / SDPbound) on one GB300.

    lib        ctypes binding of libmcbound.so (the C ABI of include/mcbound.h):
               Context.evaluate / bound_batch / bab, operator-level entry points,
               the learned models' MLP
    build      in-tree build of libmcbound.so for sm_103a
    graphs     rudy-format I/O, seeded G(n, p) and 2D torus generators, cut values
    workload   the benchmark's seeded workloads
    solve      the reference's command line: parameter file + instance -> .output report
    sharded    branch-and-bound over several ranks (one per GPU), with rebalancing
    learn      training data, training and storage of the learned models
"""
