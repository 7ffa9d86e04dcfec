"""torch front-end: see the torch sub-module."""
