set output "hist_cfg1_MOTIF00000.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-82.2835:24.1048]
set yrange [0:172664]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00000.dat" using 1:2 title 'MOTIF00000 (cfg1)' with boxes
