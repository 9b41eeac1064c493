"""CPU oracle of the qTIP4P/F force and ring-polymer propagation path.

TEST INFRASTRUCTURE ONLY (the checker of the CUDA library and the timed CPU
baseline); the product package never imports it.
"""
