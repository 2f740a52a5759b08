"""Headless stand-in for matplotlib, used only when the golden-fixture generator
runs the reference solver (whose last step plots the solution)."""
