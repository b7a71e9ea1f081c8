/* Test-infrastructure shim: empty stand-in for an MKL header the reference includes but does not use. */
