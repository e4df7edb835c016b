"""CPU oracle: a plain restatement of the reference's contact and Newton-step math.

Test infrastructure only.  The product path (libcipc.so and its Python host
layer) never imports this package.
"""
