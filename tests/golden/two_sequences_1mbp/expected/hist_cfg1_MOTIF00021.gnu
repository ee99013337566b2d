set output "hist_cfg1_MOTIF00021.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-82.1457:25.1728]
set yrange [0:174083]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00021.dat" using 1:2 title 'MOTIF00021 (cfg1)' with boxes
