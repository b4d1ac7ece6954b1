"""Monte Carlo drivers and the ``neuralce-mc`` command line (the reference's ``neuralce/mc/run.py`` interface)."""
