"""The oracle: CPU restatements of the reference's time step used to check
the device path (test infrastructure; the product never imports it)."""
