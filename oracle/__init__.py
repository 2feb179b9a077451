"""Oracle package — test infrastructure only (checker and CPU baseline).

Nothing under ``stablebear_gb300/`` imports this package.
"""
