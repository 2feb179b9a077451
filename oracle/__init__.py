"""Oracle package — test infrastructure only (parity reference and CPU baseline).

Nothing under ``stablebear_gb300/`` imports this package.
"""
