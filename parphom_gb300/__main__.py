from .driver import main

main()
